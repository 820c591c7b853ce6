// Building blocks of the learned surrogate: a U-Net over height maps, BF16
// weights and activations with FP32 accumulation, NHWC layout (channels
// innermost), zero-padded 3x3 convolutions.
//
//   k_conv3x3       y = conv3x3(x, w) + b as an implicit GEMM on the tensor
//                   cores (warp-level mma m16n8k16, bf16 in, fp32 out):
//                   rows = pixels, columns = output channels, K = 9 taps x
//                   input channels, tiles staged in shared memory and read
//                   by ldmatrix. The input gradient is the same kernel on
//                   dy with the weights flipped and transposed (k_flip).
//   k_conv_wgrad    dW += dy^T x_shifted, an implicit GEMM with K = pixels:
//                   pixel tiles staged in shared memory, fragments by
//                   ldmatrix .trans, pixel chunks reduced with fp32 atomics.
//   k_bias_grad     db += sum over pixels of dy.
//   elementwise     GELU (erf form) and its derivative, 2x2 average pooling,
//                   nearest 2x upsampling and their adjoints, adds, the
//                   input packing, the squared-error loss and Adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "swe_kernels.h"
#include "swe_nn_math.cuh"

namespace swe {
namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// D += A B for one 16x8x16 tile: A row-major 16x16, B column-major 16x8,
// bf16 operands, fp32 accumulators.
__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

constexpr int kConvNT = 4;     // output-channel tiles of 8 per warp (32 channels)
constexpr int kConvPix = 64;   // pixels per block (4 warps x 16)
constexpr int kConvK = 32;     // input channels per stage
constexpr int kConvStride = 40;  // smem row stride in bf16 (80 bytes)

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const bf16* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}

// One block: 64 pixels x 32 output channels, 4 warps of 16 pixels x 32
// channels. For every tap and 32-channel slice of the input, the block
// copies the tap-shifted input rows (64 pixels x 32 channels, zero outside
// the map) and the weights (32 output x 32 input channels) into shared
// memory with 16-byte loads; ldmatrix hands out the fragments (A: pixels x
// input channels, B: input x output channels). Requires cin % 8 == 0 and
// cout % 8 == 0.
__global__ void __launch_bounds__(128) k_conv3x3(const bf16* __restrict__ x, const bf16* __restrict__ w,
                                                 const float* __restrict__ bias, bf16* __restrict__ y, int N, int H,
                                                 int W, int cin, int cout) {
  __shared__ __align__(16) bf16 sa[kConvPix * kConvStride];
  __shared__ __align__(16) bf16 sb[8 * kConvNT * kConvStride];
  const long M = (long)N * H * W;
  const long m0 = (long)blockIdx.x * kConvPix;
  const int co0 = blockIdx.y * 8 * kConvNT;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3, mi = lane >> 3, r = lane & 7;
  // staging of A: thread -> pixel rows tid/4 and 32 + tid/4, 8-channel segment
  const int arow = tid >> 2, aseg = (tid & 3) * 8;
  long ap[2];
  int apx[2], apy[2];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    ap[h] = m0 + arow + 32 * h;
    const long pp = ap[h] < M ? ap[h] : 0;
    apx[h] = (int)(pp % W);
    apy[h] = (int)((pp / W) % H);
  }
  float acc[kConvNT][4];
#pragma unroll
  for (int j = 0; j < kConvNT; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[j][q] = 0.0f;

  for (int tap = 0; tap < 9; tap++) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    for (int c0 = 0; c0 < cin; c0 += kConvK) {
      uint4 va[2], vb = make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int h = 0; h < 2; h++) {
        va[h] = make_uint4(0, 0, 0, 0);
        const int yy = apy[h] + dy, xx = apx[h] + dx;
        if (ap[h] < M && c0 + aseg < cin && yy >= 0 && yy < H && xx >= 0 && xx < W)
          va[h] = *reinterpret_cast<const uint4*>(x + (ap[h] + (long)dy * W + dx) * cin + c0 + aseg);
      }
      if (co0 + arow < cout && c0 + aseg < cin)
        vb = *reinterpret_cast<const uint4*>(w + ((long)(co0 + arow) * 9 + tap) * cin + c0 + aseg);
      __syncthreads();  // the previous stage's fragments are read
#pragma unroll
      for (int h = 0; h < 2; h++) *reinterpret_cast<uint4*>(sa + (arow + 32 * h) * kConvStride + aseg) = va[h];
      *reinterpret_cast<uint4*>(sb + arow * kConvStride + aseg) = vb;
      __syncthreads();
#pragma unroll
      for (int k0 = 0; k0 < kConvK; k0 += 16) {
        uint32_t a0, a1, a2, a3;
        // A (16 px x 16 ci): matrices (px 0-7 | 8-15) x (ci 0-7 | 8-15)
        ldsm_x4(a0, a1, a2, a3, sa + (warp * 16 + r + ((mi & 1) << 3)) * kConvStride + k0 + ((mi >> 1) << 3));
#pragma unroll
        for (int j = 0; j < kConvNT; j += 2) {
          // B for output-channel tiles j, j+1: (co 0-7 | 8-15) x (ci 0-7 | 8-15)
          uint32_t b0, b1, b2, b3;
          ldsm_x4(b0, b1, b2, b3, sb + (8 * j + r + ((mi >> 1) << 3)) * kConvStride + k0 + ((mi & 1) << 3));
          mma16816(acc[j], a0, a1, a2, a3, b0, b1);
          mma16816(acc[j + 1], a0, a1, a2, a3, b2, b3);
        }
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kConvNT; j++) {
    const int co = co0 + 8 * j + 2 * t;
    if (co >= cout) continue;
    const float b0 = bias ? bias[co] : 0.0f, b1 = bias ? bias[co + 1] : 0.0f;
#pragma unroll
    for (int r2 = 0; r2 < 2; r2++) {
      const long p = m0 + warp * 16 + g + 8 * r2;
      if (p >= M) continue;
      const uint32_t v = pack2(__float2bfloat16_rn(acc[j][2 * r2] + b0), __float2bfloat16_rn(acc[j][2 * r2 + 1] + b1));
      *reinterpret_cast<uint32_t*>(y + p * cout + co) = v;
    }
  }
}

// wf[ci][tap][co] = w[co][8 - tap][ci]: the weights of the input-gradient
// convolution (the adjoint of a zero-padded 3x3 convolution is the
// convolution with the spatially flipped, transposed kernel).
__global__ void k_flip(const bf16* __restrict__ w, bf16* __restrict__ wf, int cin, int cout) {
  const long n = (long)cout * 9 * cin;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int ci = (int)(i % cin);
    const int tap = (int)((i / cin) % 9);
    const int co = (int)(i / (9L * cin));
    wf[((long)ci * 9 + (8 - tap)) * cout + co] = w[i];
  }
}

// Weight gradient tiles: one block = 32 output x 32 input channels of one
// tap over a chunk of pixels; 4 warps, each 16 x 16 (two 8-column mma
// tiles); pixels staged 32 at a time (two mma k-steps).
constexpr int kWgTile = 32;
constexpr int kWgPix = 32;
constexpr int kWgChunk = 4096;  // pixels per block
constexpr int kWgStride = 40;   // smem row stride in bf16 (80 bytes: 16-byte aligned rows, fewer conflicts)

__device__ __forceinline__ void ldsm_x4_trans(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3,
                                              const bf16* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}

// dW[co][tap][ci] += sum_p dy[p][co] x[p + off(tap)][ci] (zero padding).
// As a GEMM per tap: rows co, columns ci, K = pixels. One block covers all
// nine taps of a 32 x 32 (co, ci) tile, so a pixel chunk is read once per
// block: each stage copies 32 pixels of dy (32 channels from co0) and, for
// every tap, the 32 tap-shifted pixels of x (32 channels from ci0) into
// shared memory, rows = pixels, with 16-byte loads (the nine shifted copies
// overlap, so most of their reads hit L1); ldmatrix .trans then hands out
// the fragments (A = dy^T, B = x, both with pixel pairs per register).
// Channels past cout / cin and pixels past the map or the batch are zero.
// The block's 9 x 32 x 32 partial sums go to dw with fp32 atomics. Requires
// cin % 8 == 0 and cout % 8 == 0.
__global__ void __launch_bounds__(128) k_conv_wgrad(const bf16* __restrict__ x, const bf16* __restrict__ dy,
                                                    float* __restrict__ dw, int N, int H, int W, int cin, int cout) {
  __shared__ __align__(16) bf16 sdy[kWgPix * kWgStride];
  __shared__ __align__(16) bf16 sx[9 * kWgPix * kWgStride];
  const long M = (long)N * H * W;
  const int ctile = (cin + kWgTile - 1) / kWgTile;
  const int ci0 = (blockIdx.y % ctile) * kWgTile;
  const int co0 = (blockIdx.y / ctile) * kWgTile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 16, wn = (warp & 1) * 16;  // the warp's co / ci offsets in the tile
  // staging: thread -> (pixel row, 8-channel segment)
  const int srow = tid >> 2, sseg = (tid & 3) * 8;
  float acc[9][2][4];
#pragma unroll
  for (int tp = 0; tp < 9; tp++)
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[tp][j][q] = 0.0f;

  const long pbeg = (long)blockIdx.x * kWgChunk;
  const long pend = pbeg + kWgChunk < M ? pbeg + kWgChunk : M;
  for (long p0 = pbeg; p0 < pend; p0 += kWgPix) {
    const long p = p0 + srow;
    uint4 vdy = make_uint4(0, 0, 0, 0);
    uint4 vx[9];
    int px = 0, py = 0;
    if (p < pend) {
      if (co0 + sseg < cout) vdy = *reinterpret_cast<const uint4*>(dy + p * cout + co0 + sseg);
      px = (int)(p % W);
      py = (int)((p / W) % H);
    }
#pragma unroll
    for (int tp = 0; tp < 9; tp++) {
      const int ddy = tp / 3 - 1, ddx = tp % 3 - 1;
      const int xx = px + ddx, yy = py + ddy;
      vx[tp] = make_uint4(0, 0, 0, 0);
      if (p < pend && ci0 + sseg < cin && xx >= 0 && xx < W && yy >= 0 && yy < H)
        vx[tp] = *reinterpret_cast<const uint4*>(x + (p + (long)ddy * W + ddx) * cin + ci0 + sseg);
    }
    __syncthreads();  // the previous stage's fragments are read
    *reinterpret_cast<uint4*>(sdy + srow * kWgStride + sseg) = vdy;
#pragma unroll
    for (int tp = 0; tp < 9; tp++)
      *reinterpret_cast<uint4*>(sx + (tp * kWgPix + srow) * kWgStride + sseg) = vx[tp];
    __syncthreads();
    const int mi = lane >> 3, r = lane & 7;
#pragma unroll
    for (int k0 = 0; k0 < kWgPix; k0 += 16) {
      // A (16 co x 16 px): matrices (co 0-7 | 8-15) x (px 0-7 | 8-15)
      uint32_t a0, a1, a2, a3;
      ldsm_x4_trans(a0, a1, a2, a3, sdy + (k0 + r + ((mi >> 1) << 3)) * kWgStride + wm + ((mi & 1) << 3));
#pragma unroll
      for (int tp = 0; tp < 9; tp++) {
        // B (16 px x 16 ci): matrices (px 0-7 | 8-15) x (ci 0-7 | 8-15)
        uint32_t b0, b1, b2, b3;
        ldsm_x4_trans(b0, b1, b2, b3,
                      sx + (tp * kWgPix + k0 + r + ((mi & 1) << 3)) * kWgStride + wn + ((mi >> 1) << 3));
        mma16816(acc[tp][0], a0, a1, a2, a3, b0, b1);
        mma16816(acc[tp][1], a0, a1, a2, a3, b2, b3);
      }
    }
  }
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int tp = 0; tp < 9; tp++)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const int ci = ci0 + wn + 8 * j + 2 * t;
#pragma unroll
      for (int r2 = 0; r2 < 2; r2++) {
        const int co = co0 + wm + g + 8 * r2;
        if (co >= cout || ci >= cin) continue;
        float* o = dw + ((long)co * 9 + tp) * cin + ci;
        atomicAdd(o, acc[tp][j][2 * r2]);
        atomicAdd(o + 1, acc[tp][j][2 * r2 + 1]);
      }
    }
}

// db[co] += sum_p dy[p][co]. Thread -> (pixel row, 8-channel group) with
// 16-byte loads; per-thread sums go to shared-memory accumulators, then one
// global atomic per channel per block. cout % 8 == 0, cout <= 256.
__global__ void k_bias_grad(const bf16* __restrict__ dy, float* __restrict__ db, long M, int cout) {
  __shared__ float sdb[256];
  const int groups = cout / 8;
  const int rows = blockDim.x / groups;
  for (int c = threadIdx.x; c < cout; c += blockDim.x) sdb[c] = 0.0f;
  __syncthreads();
  if ((int)threadIdx.x < rows * groups) {
    const int grp = threadIdx.x % groups, row = threadIdx.x / groups;
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long p = (long)blockIdx.x * rows + row; p < M; p += (long)gridDim.x * rows) {
      const uint4 v = *reinterpret_cast<const uint4*>(dy + p * cout + grp * 8);
      const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
      for (int k = 0; k < 8; k++) acc[k] += __bfloat162float(e[k]);
    }
#pragma unroll
    for (int k = 0; k < 8; k++) atomicAdd(&sdb[grp * 8 + k], acc[k]);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < cout; c += blockDim.x) atomicAdd(db + c, sdb[c]);
}

__device__ __forceinline__ float gelu(float v) { return gelu_as(v); }
__device__ __forceinline__ float gelu_grad(float v) { return gelu_grad_as(v); }

// The elementwise kernels move 8 bf16 values (16 bytes) per thread step;
// counts and channel numbers are multiples of 8 (checked by the callers).
struct Vec8 {
  float v[8];
  __device__ __forceinline__ void load(const bf16* p) {
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    const bf16* e = reinterpret_cast<const bf16*>(&u);
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = __bfloat162float(e[k]);
  }
  __device__ __forceinline__ void store(bf16* p) const {
    uint4 u;
    bf16* e = reinterpret_cast<bf16*>(&u);
#pragma unroll
    for (int k = 0; k < 8; k++) e[k] = __float2bfloat16_rn(v[k]);
    *reinterpret_cast<uint4*>(p) = u;
  }
};

__global__ void k_gelu(const bf16* __restrict__ pre, bf16* __restrict__ act, long n8) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n8; i += (long)gridDim.x * blockDim.x) {
    Vec8 a;
    a.load(pre + 8 * i);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] = gelu(a.v[k]);
    a.store(act + 8 * i);
  }
}

__global__ void k_gelu_bwd(const bf16* __restrict__ pre, const bf16* __restrict__ dact, bf16* __restrict__ dpre,
                           long n8) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n8; i += (long)gridDim.x * blockDim.x) {
    Vec8 a, d;
    a.load(pre + 8 * i);
    d.load(dact + 8 * i);
#pragma unroll
    for (int k = 0; k < 8; k++) d.v[k] = d.v[k] * gelu_grad(a.v[k]);
    d.store(dpre + 8 * i);
  }
}

// y[n][i][j][c] = mean of x[n][2i..2i+1][2j..2j+1][c] (H, W even: the input's).
template <class I>
__global__ void k_pool2(const bf16* __restrict__ x, bf16* __restrict__ y, int N, int H, int W, int C) {
  const int Ho = H / 2, Wo = W / 2, G = C / 8;
  const I n = (I)N * Ho * Wo * G;
  for (I i = blockIdx.x * (I)blockDim.x + threadIdx.x; i < n; i += (I)gridDim.x * blockDim.x) {
    const int c = (int)(i % G) * 8;
    const I q = i / G;
    const int j = (int)(q % Wo), ii = (int)((q / Wo) % Ho);
    const I b = q / ((I)Wo * Ho);
    const I s = ((b * H + 2 * ii) * W + 2 * j) * C + c;
    Vec8 a, t;
    a.load(x + s);
    t.load(x + s + C);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] += t.v[k];
    t.load(x + s + (I)W * C);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] += t.v[k];
    t.load(x + s + (I)W * C + C);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] = 0.25f * (a.v[k] + t.v[k]);
    a.store(y + q * C + c);
  }
}

// dx[n][y][x][c] = dy[n][y/2][x/2][c] / 4 (H, W: the pooling's input).
template <class I>
__global__ void k_pool2_bwd(const bf16* __restrict__ dy, bf16* __restrict__ dx, int N, int H, int W, int C) {
  const int G = C / 8;
  const I n = (I)N * H * W * G;
  for (I i = blockIdx.x * (I)blockDim.x + threadIdx.x; i < n; i += (I)gridDim.x * blockDim.x) {
    const int c = (int)(i % G) * 8;
    const I q = i / G;
    const int xx = (int)(q % W), yy = (int)((q / W) % H);
    const I b = q / ((I)W * H);
    Vec8 a;
    a.load(dy + ((b * (H / 2) + yy / 2) * (W / 2) + xx / 2) * C + c);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] *= 0.25f;
    a.store(dx + q * C + c);
  }
}

// y[n][y][x][c] = x[n][y/2][x/2][c] (H, W: the input's; the output is 2H x 2W).
template <class I>
__global__ void k_up2(const bf16* __restrict__ x, bf16* __restrict__ y, int N, int H, int W, int C) {
  const int Ho = 2 * H, Wo = 2 * W, G = C / 8;
  const I n = (I)N * Ho * Wo * G;
  for (I i = blockIdx.x * (I)blockDim.x + threadIdx.x; i < n; i += (I)gridDim.x * blockDim.x) {
    const int c = (int)(i % G) * 8;
    const I q = i / G;
    const int xx = (int)(q % Wo), yy = (int)((q / Wo) % Ho);
    const I b = q / ((I)Wo * Ho);
    *reinterpret_cast<uint4*>(y + q * C + c) =
        *reinterpret_cast<const uint4*>(x + ((b * H + yy / 2) * W + xx / 2) * C + c);
  }
}

// dx[n][i][j][c] = sum of dy over the 2x2 block (H, W: the upsampling's input).
template <class I>
__global__ void k_up2_bwd(const bf16* __restrict__ dy, bf16* __restrict__ dx, int N, int H, int W, int C) {
  const int G = C / 8, Wo = 2 * W;
  const I n = (I)N * H * W * G;
  for (I i = blockIdx.x * (I)blockDim.x + threadIdx.x; i < n; i += (I)gridDim.x * blockDim.x) {
    const int c = (int)(i % G) * 8;
    const I q = i / G;
    const int j = (int)(q % W), ii = (int)((q / W) % H);
    const I b = q / ((I)W * H);
    const I s = ((b * 2 * H + 2 * ii) * Wo + 2 * j) * C + c;
    Vec8 a, t;
    a.load(dy + s);
    t.load(dy + s + C);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] += t.v[k];
    t.load(dy + s + (I)Wo * C);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] += t.v[k];
    t.load(dy + s + (I)Wo * C + C);
#pragma unroll
    for (int k = 0; k < 8; k++) a.v[k] += t.v[k];
    a.store(dx + q * C + c);
  }
}

__global__ void k_add(const bf16* __restrict__ a, const bf16* __restrict__ b, bf16* __restrict__ out, long n8) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n8; i += (long)gridDim.x * blockDim.x) {
    Vec8 u, v;
    u.load(a + 8 * i);
    v.load(b + 8 * i);
#pragma unroll
    for (int k = 0; k < 8; k++) u.v[k] += v.v[k];
    u.store(out + 8 * i);
  }
}

// Network input, 16 channels per pixel: (height - 0.25) * 4, the wind
// direction's x and z components, zeros.
// With means (per map, device), the heights are first moved so that each
// map's mean is `ref`: ((h - mean) + (ref - 0.25)) * 4. A pixel's 16
// channels (32 bytes) leave in two 16-byte stores where x is 16-byte aligned.
__global__ void k_pack_input(const float* __restrict__ h, const float* __restrict__ wind_xz, bf16* __restrict__ x,
                             int N, int H, int W, const float* __restrict__ means, float ref, bool vec) {
  const long n = (long)N * H * W;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
    const long b = p / ((long)H * W);
    const bf16 c0 = __float2bfloat16_rn(means ? ((h[p] - means[b]) + (ref - 0.25f)) * 4.0f : (h[p] - 0.25f) * 4.0f);
    const bf16 c1 = __float2bfloat16_rn(wind_xz[2 * b]);
    const bf16 c2 = __float2bfloat16_rn(wind_xz[2 * b + 1]);
    bf16* o = x + p * 16;
    if (vec) {
      const uint32_t w0 = (uint32_t)__bfloat16_as_ushort(c0) | ((uint32_t)__bfloat16_as_ushort(c1) << 16);
      const uint32_t w1 = (uint32_t)__bfloat16_as_ushort(c2);
      reinterpret_cast<uint4*>(o)[0] = make_uint4(w0, w1, 0u, 0u);
      reinterpret_cast<uint4*>(o)[1] = make_uint4(0u, 0u, 0u, 0u);
    } else {
      o[0] = c0;
      o[1] = c1;
      o[2] = c2;
#pragma unroll
      for (int c = 3; c < 16; c++) o[c] = __float2bfloat16_rn(0.0f);
    }
  }
}

// Squared-error loss on channel 0 of pred (C channels) against target *
// tscale: sum of squares into *loss, d pred = 2 (pred - target tscale)
// gscale on channel 0, zero elsewhere.
// With vec (C a multiple of 8, dpred 16-byte aligned) a pixel's gradient
// leaves in C / 8 16-byte stores.
__global__ void k_mse(const bf16* __restrict__ pred, const float* __restrict__ target, float tscale,
                      bf16* __restrict__ dpred, float* __restrict__ loss, long M, int C, float scale, bool vec) {
  float s = 0.0f;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < M; p += (long)gridDim.x * blockDim.x) {
    const float e = __bfloat162float(pred[p * C]) - target[p] * tscale;
    s += e * e;
    const bf16 d0 = __float2bfloat16_rn(2.0f * e * scale);
    if (vec) {
      uint4* o = reinterpret_cast<uint4*>(dpred + p * C);
      o[0] = make_uint4((uint32_t)__bfloat16_as_ushort(d0), 0u, 0u, 0u);
      for (int c = 1; c < C / 8; c++) o[c] = make_uint4(0u, 0u, 0u, 0u);
    } else {
      dpred[p * C] = d0;
      for (int c = 1; c < C; c++) dpred[p * C + c] = __float2bfloat16_rn(0.0f);
    }
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

// Channel 0 of pred as floats, times oscale.
__global__ void k_channel0(const bf16* __restrict__ pred, float* __restrict__ out, long M, int C, float oscale) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < M; p += (long)gridDim.x * blockDim.x)
    out[p] = __bfloat162float(pred[p * C]) * oscale;
}

// Adam (Kingma & Ba, 2015) on fp32 master weights, with the bf16 copy the
// kernels read.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, bf16* __restrict__ w16, long n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float gr = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gr;
    const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
  }
}

__global__ void k_to_bf16(const float* __restrict__ a, bf16* __restrict__ b, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}

inline unsigned grid_for(long n, int threads = 256) {
  long g = (n + threads - 1) / threads;
  if (g > 152L * 32) g = 152L * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t nn_conv3x3(const void* x, const void* w, const float* bias, void* y, int N, int H, int W, int cin,
                       int cout, cudaStream_t s) {
  const long M = (long)N * H * W;
  const long blocks = (M + kConvPix - 1) / kConvPix;
  const int cblocks = (cout + 8 * kConvNT - 1) / (8 * kConvNT);
  if (blocks > 0x7fffffffL || cblocks > 65535) return cudaErrorInvalidValue;
  k_conv3x3<<<dim3((unsigned)blocks, (unsigned)cblocks), 128, 0, s>>>(
      static_cast<const bf16*>(x), static_cast<const bf16*>(w), bias, static_cast<bf16*>(y), N, H, W, cin, cout);
  return cudaGetLastError();
}

cudaError_t nn_flip(const void* w, void* wf, int cin, int cout, cudaStream_t s) {
  k_flip<<<grid_for((long)cout * 9 * cin), 256, 0, s>>>(static_cast<const bf16*>(w), static_cast<bf16*>(wf), cin,
                                                       cout);
  return cudaGetLastError();
}

cudaError_t nn_conv_wgrad(const void* x, const void* dy, float* dw, float* db, int N, int H, int W, int cin, int cout,
                          cudaStream_t s) {
  const long M = (long)N * H * W;
  const long chunks = (M + kWgChunk - 1) / kWgChunk;
  const int tiles = ((cin + kWgTile - 1) / kWgTile) * ((cout + kWgTile - 1) / kWgTile);
  if (chunks > 0x7fffffffL || tiles > 65535) return cudaErrorInvalidValue;
  k_conv_wgrad<<<dim3((unsigned)chunks, (unsigned)tiles), 128, 0, s>>>(static_cast<const bf16*>(x),
                                                                      static_cast<const bf16*>(dy), dw, N, H, W, cin,
                                                                      cout);
  if (db) {
    long bx = (M + 255) / 256;
    if (bx > 1024) bx = 1024;
    k_bias_grad<<<(unsigned)bx, 256, 0, s>>>(static_cast<const bf16*>(dy), db, M, cout);
  }
  return cudaGetLastError();
}

cudaError_t nn_bias_grad(const void* dy, float* db, long M, int cout, cudaStream_t s) {
  long bx = (M + 255) / 256;
  if (bx > 1024) bx = 1024;
  k_bias_grad<<<(unsigned)bx, 256, 0, s>>>(static_cast<const bf16*>(dy), db, M, cout);
  return cudaGetLastError();
}

cudaError_t nn_gelu(const void* pre, void* act, long n, cudaStream_t s) {
  k_gelu<<<grid_for(n / 8), 256, 0, s>>>(static_cast<const bf16*>(pre), static_cast<bf16*>(act), n / 8);
  return cudaGetLastError();
}

cudaError_t nn_gelu_bwd(const void* pre, const void* dact, void* dpre, long n, cudaStream_t s) {
  k_gelu_bwd<<<grid_for(n / 8), 256, 0, s>>>(static_cast<const bf16*>(pre), static_cast<const bf16*>(dact),
                                             static_cast<bf16*>(dpre), n / 8);
  return cudaGetLastError();
}

// 32-bit index arithmetic (its divisions are several times cheaper than
// 64-bit ones) whenever every element index fits.
constexpr long kIndex32 = 0x7fffffffL;

cudaError_t nn_pool2(const void* x, void* y, int N, int H, int W, int C, bool backward, cudaStream_t s) {
  const long n = (long)N * H * W * C;
  const bf16* in = static_cast<const bf16*>(x);
  bf16* out = static_cast<bf16*>(y);
  if (backward) {
    if (4 * n <= kIndex32)
      k_pool2_bwd<int><<<grid_for(n / 8), 256, 0, s>>>(in, out, N, H, W, C);
    else
      k_pool2_bwd<long><<<grid_for(n / 8), 256, 0, s>>>(in, out, N, H, W, C);
  } else {
    if (n <= kIndex32)
      k_pool2<int><<<grid_for(n / 32), 256, 0, s>>>(in, out, N, H, W, C);
    else
      k_pool2<long><<<grid_for(n / 32), 256, 0, s>>>(in, out, N, H, W, C);
  }
  return cudaGetLastError();
}

cudaError_t nn_up2(const void* x, void* y, int N, int H, int W, int C, bool backward, cudaStream_t s) {
  const long n = (long)N * H * W * C;
  const bf16* in = static_cast<const bf16*>(x);
  bf16* out = static_cast<bf16*>(y);
  if (backward) {
    if (4 * n <= kIndex32)
      k_up2_bwd<int><<<grid_for(n / 8), 256, 0, s>>>(in, out, N, H, W, C);
    else
      k_up2_bwd<long><<<grid_for(n / 8), 256, 0, s>>>(in, out, N, H, W, C);
  } else {
    if (4 * n <= kIndex32)
      k_up2<int><<<grid_for(n / 2), 256, 0, s>>>(in, out, N, H, W, C);
    else
      k_up2<long><<<grid_for(n / 2), 256, 0, s>>>(in, out, N, H, W, C);
  }
  return cudaGetLastError();
}

cudaError_t nn_add(const void* a, const void* b, void* out, long n, cudaStream_t s) {
  k_add<<<grid_for(n / 8), 256, 0, s>>>(static_cast<const bf16*>(a), static_cast<const bf16*>(b),
                                        static_cast<bf16*>(out), n / 8);
  return cudaGetLastError();
}

// Mean of each of N maps of M floats, one CTA per map: per-thread float
// partial sums in a fixed order, then a fixed-order block reduction in
// double (the same result on every run).
__global__ void __launch_bounds__(1024) k_map_mean(const float* __restrict__ h, long M, float* __restrict__ means) {
  __shared__ double part[32];
  const float* m = h + (long)blockIdx.x * M;
  float acc = 0.0f;
  for (long i = threadIdx.x; i < M; i += blockDim.x) acc += m[i];
  double d = acc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
    means[blockIdx.x] = (float)(t / (double)M);
  }
}

cudaError_t nn_pack_input(const float* h, const float* wind_xz, void* x, int N, int H, int W, cudaStream_t s,
                          float* means, float ref) {
  if (means) k_map_mean<<<N, 1024, 0, s>>>(h, (long)H * W, means);
  const bool vec = (reinterpret_cast<uintptr_t>(x) & 15) == 0;
  k_pack_input<<<grid_for((long)N * H * W), 256, 0, s>>>(h, wind_xz, static_cast<bf16*>(x), N, H, W, means, ref, vec);
  return cudaGetLastError();
}

cudaError_t nn_mse(const void* pred, const float* target, float tscale, void* dpred, float* loss, long M, int C,
                   float gscale, cudaStream_t s) {
  const bool vec = C % 8 == 0 && (reinterpret_cast<uintptr_t>(dpred) & 15) == 0;
  k_mse<<<grid_for(M), 256, 0, s>>>(static_cast<const bf16*>(pred), target, tscale, static_cast<bf16*>(dpred), loss,
                                    M, C, gscale, vec);
  return cudaGetLastError();
}

cudaError_t nn_channel0(const void* pred, float* out, long M, int C, float oscale, cudaStream_t s) {
  k_channel0<<<grid_for(M), 256, 0, s>>>(static_cast<const bf16*>(pred), out, M, C, oscale);
  return cudaGetLastError();
}

cudaError_t nn_adam(float* w, const float* grad, float* m, float* v, void* w16, long n, float lr, float b1, float b2,
                    float eps, int step, cudaStream_t s) {
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_adam<<<grid_for(n), 256, 0, s>>>(w, grad, m, v, static_cast<bf16*>(w16), n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t nn_to_bf16(const float* a, void* b, long n, cudaStream_t s) {
  k_to_bf16<<<grid_for(n), 256, 0, s>>>(a, static_cast<bf16*>(b), n);
  return cudaGetLastError();
}

}  // namespace swe

// ---- C ABI (include/swe.h): argument checks, then the launch ----
#include <string>

#include "swe.h"

namespace {

int nn_fail(int code, const std::string& msg) {
  swe::set_last_error(msg);
  return code;
}

int nn_done(cudaError_t e) {
  if (e != cudaSuccess) return nn_fail(SWE_ERR_CUDA, cudaGetErrorString(e));
  return SWE_OK;
}

bool aligned4(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; }
bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" {

int swe_nn_conv3x3(const void* x, const void* w, const float* bias, void* y, int n, int h, int wd, int cin, int cout,
                   void* stream) {
  if (!x || !w || !y) return nn_fail(SWE_ERR_INVALID, "NULL tensor");
  if (n < 1 || h < 1 || wd < 1 || cin < 16 || cin % 16 || cout < 8 || cout % 8)
    return nn_fail(SWE_ERR_INVALID, "conv3x3: need n, h, w >= 1, cin % 16 == 0, cout % 8 == 0");
  if (!aligned16(x) || !aligned16(w) || !aligned4(y))
    return nn_fail(SWE_ERR_INVALID, "x and w must be 16-byte aligned, y 4-byte aligned");
  return nn_done(swe::nn_conv3x3(x, w, bias, y, n, h, wd, cin, cout, static_cast<cudaStream_t>(stream)));
}

int swe_nn_conv3x3_tc_pack(const void* w, void* wp, int cin, int cout, int flip, void* stream) {
  if (!w || !wp || cin < 1 || cout < 1) return nn_fail(SWE_ERR_INVALID, "conv3x3_tc_pack: bad arguments");
  return nn_done(swe::nn_pack_tc(w, wp, cin, cout, flip != 0, static_cast<cudaStream_t>(stream)));
}

int swe_nn_conv3x3_tc(const void* x, const void* wp, const float* bias, void* y, void* act, int n, int h, int wd,
                      int cin, int cout, void* stream) {
  if (!x || !wp || !y) return nn_fail(SWE_ERR_INVALID, "NULL tensor");
  if (n < 1 || !swe::nn_conv_tc_supported(h, wd, cin, cout))
    return nn_fail(SWE_ERR_INVALID,
                   "conv3x3_tc: need cin % 16 == 0, cout % 16 == 0, cout <= 256, a width with a power-of-two "
                   "factor TW >= 8 (up to 128) and a height that is a multiple of 128 / TW");
  if (!aligned16(x) || !aligned16(wp) || !aligned16(y) || (act && !aligned16(act)))
    return nn_fail(SWE_ERR_INVALID, "conv3x3_tc: tensors must be 16-byte aligned");
  return nn_done(swe::nn_conv_tc(x, wp, bias, y, act, n, h, wd, cin, cout, static_cast<cudaStream_t>(stream)));
}

int swe_nn_conv3x3_wgrad_tc(const void* x, const void* dy, float* dw, float* db, int n, int h, int wd, int cin,
                            int cout, void* stream) {
  if (!x || !dy || !dw) return nn_fail(SWE_ERR_INVALID, "NULL tensor");
  if (n < 1 || !swe::nn_wgrad_tc_supported(h, wd, cin, cout))
    return nn_fail(SWE_ERR_INVALID,
                   "conv3x3_wgrad_tc: need cin, cout multiples of 16 up to 128, a width with a power-of-two "
                   "factor TW >= 8 (up to 128) and a height that is a multiple of 128 / TW");
  if (!aligned16(x) || !aligned16(dy)) return nn_fail(SWE_ERR_INVALID, "tensors must be 16-byte aligned");
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return nn_fail(SWE_ERR_CUDA, "no current device");
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  return nn_done(swe::nn_wgrad_tc(x, dy, dw, db, n, h, wd, cin, cout, sms, s));
}

int swe_nn_status(uint32_t* status) {
  unsigned int v = 0;
  if (int rc = nn_done(swe::nn_tc_status(&v))) return rc;
  if (status) *status = v;
  if (v) return nn_fail(SWE_ERR_DEVICE, "a tensor-core kernel gave up waiting (code " + std::to_string(v) + ")");
  return SWE_OK;
}

int swe_nn_conv3x3_flip(const void* w, void* wf, int cin, int cout, void* stream) {
  if (!w || !wf || cin < 1 || cout < 1) return nn_fail(SWE_ERR_INVALID, "conv3x3_flip: bad arguments");
  return nn_done(swe::nn_flip(w, wf, cin, cout, static_cast<cudaStream_t>(stream)));
}

int swe_nn_conv3x3_wgrad(const void* x, const void* dy, float* dw, float* db, int n, int h, int wd, int cin, int cout,
                         void* stream) {
  if (!x || !dy || !dw) return nn_fail(SWE_ERR_INVALID, "NULL tensor");
  if (n < 1 || h < 1 || wd < 1 || cin < 16 || cin % 16 || cout < 8 || cout % 8 || cout > 256)
    return nn_fail(SWE_ERR_INVALID, "conv3x3_wgrad: need n, h, w >= 1, cin % 16 == 0, cout % 8 == 0, cout <= 256");
  if (!aligned16(x) || !aligned16(dy)) return nn_fail(SWE_ERR_INVALID, "tensors must be 16-byte aligned");
  return nn_done(swe::nn_conv_wgrad(x, dy, dw, db, n, h, wd, cin, cout, static_cast<cudaStream_t>(stream)));
}

int swe_nn_gelu(const void* pre, void* act, int64_t count, void* stream) {
  if (!pre || !act || count < 0 || count % 8 || !aligned16(pre) || !aligned16(act))
    return nn_fail(SWE_ERR_INVALID, "gelu: need count % 8 == 0 and 16-byte aligned tensors");
  if (count == 0) return SWE_OK;
  return nn_done(swe::nn_gelu(pre, act, (long)count, static_cast<cudaStream_t>(stream)));
}

int swe_nn_gelu_bwd(const void* pre, const void* dact, void* dpre, int64_t count, void* stream) {
  if (!pre || !dact || !dpre || count < 0 || count % 8 || !aligned16(pre) || !aligned16(dact) || !aligned16(dpre))
    return nn_fail(SWE_ERR_INVALID, "gelu_bwd: need count % 8 == 0 and 16-byte aligned tensors");
  if (count == 0) return SWE_OK;
  return nn_done(swe::nn_gelu_bwd(pre, dact, dpre, (long)count, static_cast<cudaStream_t>(stream)));
}

int swe_nn_pool2(const void* x, void* y, int n, int h, int wd, int c, int backward, void* stream) {
  if (!x || !y || n < 1 || h < 2 || wd < 2 || h % 2 || wd % 2 || c < 8 || c % 8 || !aligned16(x) || !aligned16(y))
    return nn_fail(SWE_ERR_INVALID, "pool2: need even h, w >= 2, c % 8 == 0, 16-byte aligned tensors");
  return nn_done(swe::nn_pool2(x, y, n, h, wd, c, backward != 0, static_cast<cudaStream_t>(stream)));
}

int swe_nn_up2(const void* x, void* y, int n, int h, int wd, int c, int backward, void* stream) {
  if (!x || !y || n < 1 || h < 1 || wd < 1 || c < 8 || c % 8 || !aligned16(x) || !aligned16(y))
    return nn_fail(SWE_ERR_INVALID, "up2: need c % 8 == 0 and 16-byte aligned tensors");
  return nn_done(swe::nn_up2(x, y, n, h, wd, c, backward != 0, static_cast<cudaStream_t>(stream)));
}

int swe_nn_add(const void* a, const void* b, void* out, int64_t count, void* stream) {
  if (!a || !b || !out || count < 0 || count % 8 || !aligned16(a) || !aligned16(b) || !aligned16(out))
    return nn_fail(SWE_ERR_INVALID, "add: need count % 8 == 0 and 16-byte aligned tensors");
  if (count == 0) return SWE_OK;
  return nn_done(swe::nn_add(a, b, out, (long)count, static_cast<cudaStream_t>(stream)));
}

int swe_nn_pack_input(const float* height, const float* wind_xz, void* x, int n, int h, int wd, void* stream) {
  if (!height || !wind_xz || !x || n < 1 || h < 1 || wd < 1) return nn_fail(SWE_ERR_INVALID, "pack_input: bad arguments");
  return nn_done(swe::nn_pack_input(height, wind_xz, x, n, h, wd, static_cast<cudaStream_t>(stream), nullptr, 0.0f));
}

int swe_nn_pack_input_centered(const float* height, const float* wind_xz, float* means, void* x, int n, int h, int wd,
                               float ref, void* stream) {
  if (!height || !wind_xz || !means || !x || n < 1 || h < 1 || wd < 1 || !(ref == ref))
    return nn_fail(SWE_ERR_INVALID, "pack_input_centered: bad arguments");
  return nn_done(swe::nn_pack_input(height, wind_xz, x, n, h, wd, static_cast<cudaStream_t>(stream), means, ref));
}

int swe_nn_mse(const void* pred, const float* target, float target_scale, void* dpred, float* loss, int64_t pixels,
               int c, float grad_scale, void* stream) {
  if (!pred || !target || !dpred || !loss || pixels < 1 || c < 1) return nn_fail(SWE_ERR_INVALID, "mse: bad arguments");
  return nn_done(swe::nn_mse(pred, target, target_scale, dpred, loss, (long)pixels, c, grad_scale,
                             static_cast<cudaStream_t>(stream)));
}

int swe_nn_channel0(const void* pred, float* out, int64_t pixels, int c, float out_scale, void* stream) {
  if (!pred || !out || pixels < 1 || c < 1) return nn_fail(SWE_ERR_INVALID, "channel0: bad arguments");
  return nn_done(swe::nn_channel0(pred, out, (long)pixels, c, out_scale, static_cast<cudaStream_t>(stream)));
}

int swe_nn_adam(float* w, const float* grad, float* m, float* v, void* w_bf16, int64_t count, float lr, float beta1,
                float beta2, float eps, int step, void* stream) {
  if (!w || !grad || !m || !v || count < 1 || step < 1) return nn_fail(SWE_ERR_INVALID, "adam: bad arguments");
  return nn_done(swe::nn_adam(w, grad, m, v, w_bf16, (long)count, lr, beta1, beta2, eps, step,
                              static_cast<cudaStream_t>(stream)));
}

int swe_nn_to_bf16(const float* a, void* b, int64_t count, void* stream) {
  if (!a || !b || count < 0) return nn_fail(SWE_ERR_INVALID, "to_bf16: bad arguments");
  if (count == 0) return SWE_OK;
  return nn_done(swe::nn_to_bf16(a, b, (long)count, static_cast<cudaStream_t>(stream)));
}

}  // extern "C"
