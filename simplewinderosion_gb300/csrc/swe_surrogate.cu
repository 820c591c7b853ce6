// Building blocks of the learned surrogate: a U-Net over height maps, BF16
// weights and activations with FP32 accumulation, NHWC layout (channels
// innermost), zero-padded 3x3 convolutions.
//
//   k_conv3x3       y = conv3x3(x, w) + b as an implicit GEMM on the tensor
//                   cores (warp-level mma m16n8k16, bf16 in, fp32 out):
//                   rows = pixels, columns = output channels, K = 9 taps x
//                   input channels. The input gradient is the same kernel on
//                   dy with the weights flipped and transposed (k_flip).
//   k_conv_wgrad    dW += dy^T x_shifted, an implicit GEMM with K = pixels,
//                   split over pixel chunks and reduced with fp32 atomics.
//   k_bias_grad     db += sum over pixels of dy.
//   elementwise     GELU (erf form) and its derivative, 2x2 average pooling,
//                   nearest 2x upsampling and their adjoints, adds, the
//                   input packing, the squared-error loss and Adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "swe_kernels.h"

namespace swe {
namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint32_t ld_pair(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

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

constexpr int kConvNT = 4;  // output-channel tiles of 8 per warp

// One warp: 16 pixels x 32 output channels. Lane (g = lane/4, t = lane%4)
// holds rows g and g+8 of the pixel tile and columns 2t, 2t+1 of each
// 8-channel tile. Requires cin % 16 == 0 and cout % 8 == 0.
__global__ void __launch_bounds__(128) k_conv3x3(const bf16* __restrict__ x, const bf16* __restrict__ w,
                                                 const float* __restrict__ bias, bf16* __restrict__ y, int N, int H,
                                                 int W, int cin, int cout) {
  const long M = (long)N * H * W;
  const long mtiles = (M + 15) / 16;
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int cblocks = (cout + 8 * kConvNT - 1) / (8 * kConvNT);
  if (warp >= mtiles * cblocks) return;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long m0 = (warp % mtiles) * 16;
  const int co0 = (int)(warp / mtiles) * 8 * kConvNT;

  long pr[2];
  int py[2], px[2];
  bool in[2];
#pragma unroll
  for (int r = 0; r < 2; r++) {
    pr[r] = m0 + g + 8 * r;
    in[r] = pr[r] < M;
    const long p = in[r] ? pr[r] : 0;
    px[r] = (int)(p % W);
    py[r] = (int)((p / W) % H);
  }
  float acc[kConvNT][4];
#pragma unroll
  for (int j = 0; j < kConvNT; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[j][q] = 0.0f;

  for (int tap = 0; tap < 9; tap++) {
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const bf16* src[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int yy = py[r] + dy, xx = px[r] + dx;
      const bool ok = in[r] && yy >= 0 && yy < H && xx >= 0 && xx < W;
      src[r] = ok ? x + (pr[r] + (long)dy * W + dx) * cin : nullptr;
    }
    for (int ci0 = 0; ci0 < cin; ci0 += 16) {
      const uint32_t a0 = src[0] ? ld_pair(src[0] + ci0 + 2 * t) : 0u;
      const uint32_t a1 = src[1] ? ld_pair(src[1] + ci0 + 2 * t) : 0u;
      const uint32_t a2 = src[0] ? ld_pair(src[0] + ci0 + 2 * t + 8) : 0u;
      const uint32_t a3 = src[1] ? ld_pair(src[1] + ci0 + 2 * t + 8) : 0u;
#pragma unroll
      for (int j = 0; j < kConvNT; j++) {
        const int co = co0 + 8 * j + g;
        uint32_t b0 = 0u, b1 = 0u;
        if (co < cout) {
          const bf16* wp = w + ((long)co * 9 + tap) * cin + ci0 + 2 * t;
          b0 = ld_pair(wp);
          b1 = ld_pair(wp + 8);
        }
        mma16816(acc[j], a0, a1, a2, a3, b0, b1);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kConvNT; j++) {
    const int co = co0 + 8 * j + 2 * t;
    if (co >= cout) continue;
    const float b0 = bias ? bias[co] : 0.0f, b1 = bias ? bias[co + 1] : 0.0f;
#pragma unroll
    for (int r = 0; r < 2; r++) {
      if (!in[r]) continue;
      const uint32_t v = pack2(__float2bfloat16_rn(acc[j][2 * r] + b0), __float2bfloat16_rn(acc[j][2 * r + 1] + b1));
      *reinterpret_cast<uint32_t*>(y + pr[r] * cout + co) = v;
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

constexpr int kWgNT = 2;        // 8-column tiles (tap, input channel) per warp
constexpr int kWgChunk = 256;   // pixels per warp (16 mma k-steps)

__device__ __forceinline__ bf16 ld_bf16(const bf16* p) { return *p; }

// dW[co][tap][ci] += sum_p dy[p][co] x[p + off(tap)][ci]: rows = output
// channels (16 per warp), columns = (tap, ci) (8 kWgNT per warp, within one
// tap since cin % 16 == 0), K = a chunk of kWgChunk pixels.
__global__ void __launch_bounds__(128) k_conv_wgrad(const bf16* __restrict__ x, const bf16* __restrict__ dy,
                                                    float* __restrict__ dw, int N, int H, int W, int cin, int cout) {
  const long M = (long)N * H * W;
  const long chunks = (M + kWgChunk - 1) / kWgChunk;
  const int rtiles = (cout + 15) / 16;
  const int ctiles = (9 * cin) / (8 * kWgNT);
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  if (warp >= chunks * rtiles * ctiles) return;
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long chunk = warp % chunks;
  const int rt = (int)((warp / chunks) % rtiles);
  const int ct = (int)(warp / (chunks * rtiles));
  const int co_a = rt * 16 + g, co_b = co_a + 8;
  float acc[kWgNT][4];
#pragma unroll
  for (int j = 0; j < kWgNT; j++)
#pragma unroll
    for (int q = 0; q < 4; q++) acc[j][q] = 0.0f;
  const bf16 zero = __float2bfloat16_rn(0.0f);

  for (int k0 = 0; k0 < kWgChunk; k0 += 16) {
    // the four pixels of this lane in the k-step: 2t, 2t+1, 2t+8, 2t+9
    long p[4];
    bool pin[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      p[q] = chunk * kWgChunk + k0 + 2 * t + (q & 1) + 8 * (q >> 1);
      pin[q] = p[q] < M;
    }
    bf16 va[4], vb[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      va[q] = (pin[q] && co_a < cout) ? ld_bf16(dy + p[q] * cout + co_a) : zero;
      vb[q] = (pin[q] && co_b < cout) ? ld_bf16(dy + p[q] * cout + co_b) : zero;
    }
    const uint32_t a0 = pack2(va[0], va[1]), a1 = pack2(vb[0], vb[1]);
    const uint32_t a2 = pack2(va[2], va[3]), a3 = pack2(vb[2], vb[3]);
#pragma unroll
    for (int j = 0; j < kWgNT; j++) {
      const int col = (ct * kWgNT + j) * 8 + g;  // (tap, ci) column of this lane
      const int tap = col / cin, ci = col % cin;
      const int ddy = tap / 3 - 1, ddx = tap % 3 - 1;
      bf16 vx[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        bool ok = pin[q];
        long src = 0;
        if (ok) {
          const int xx = (int)(p[q] % W) + ddx, yy = (int)((p[q] / W) % H) + ddy;
          ok = xx >= 0 && xx < W && yy >= 0 && yy < H;
          src = p[q] + (long)ddy * W + ddx;
        }
        vx[q] = ok ? ld_bf16(x + src * cin + ci) : zero;
      }
      mma16816(acc[j], a0, a1, a2, a3, pack2(vx[0], vx[1]), pack2(vx[2], vx[3]));
    }
  }
#pragma unroll
  for (int j = 0; j < kWgNT; j++) {
    const int col = (ct * kWgNT + j) * 8 + 2 * t;
#pragma unroll
    for (int r = 0; r < 2; r++) {
      const int co = r ? co_b : co_a;
      if (co >= cout) continue;
      // dw layout [co][tap][ci] = [co][col]
      atomicAdd(dw + (long)co * 9 * cin + col, acc[j][2 * r]);
      atomicAdd(dw + (long)co * 9 * cin + col + 1, acc[j][2 * r + 1]);
    }
  }
}

// db[co] += sum_p dy[p][co]: each thread sums a strided run of pixels of one
// channel, one atomic per thread.
__global__ void k_bias_grad(const bf16* __restrict__ dy, float* __restrict__ db, long M, int cout) {
  const int co = blockIdx.y;
  float s = 0.0f;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < M; p += (long)gridDim.x * blockDim.x)
    s += __bfloat162float(dy[p * cout + co]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(db + co, s);
}

__device__ __forceinline__ float gelu(float v) { return 0.5f * v * (1.0f + erff(v * 0.70710678f)); }
__device__ __forceinline__ float gelu_grad(float v) {
  return 0.5f * (1.0f + erff(v * 0.70710678f)) + v * 0.39894228f * expf(-0.5f * v * v);
}

__global__ void k_gelu(const bf16* __restrict__ pre, bf16* __restrict__ act, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    act[i] = __float2bfloat16_rn(gelu(__bfloat162float(pre[i])));
}

__global__ void k_gelu_bwd(const bf16* __restrict__ pre, const bf16* __restrict__ dact, bf16* __restrict__ dpre,
                           long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dpre[i] = __float2bfloat16_rn(__bfloat162float(dact[i]) * gelu_grad(__bfloat162float(pre[i])));
}

// y[n][i][j][c] = mean of x[n][2i..2i+1][2j..2j+1][c] (H, W even: the input's).
__global__ void k_pool2(const bf16* __restrict__ x, bf16* __restrict__ y, int N, int H, int W, int C) {
  const int Ho = H / 2, Wo = W / 2;
  const long n = (long)N * Ho * Wo * C;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long q = i / C;
    const int j = (int)(q % Wo), ii = (int)((q / Wo) % Ho);
    const long b = q / ((long)Wo * Ho);
    const long s = ((b * H + 2 * ii) * W + 2 * j) * C + c;
    const float v = __bfloat162float(x[s]) + __bfloat162float(x[s + C]) + __bfloat162float(x[s + (long)W * C]) +
                    __bfloat162float(x[s + (long)W * C + C]);
    y[i] = __float2bfloat16_rn(0.25f * v);
  }
}

// dx[n][y][x][c] = dy[n][y/2][x/2][c] / 4 (H, W: the pooling's input).
__global__ void k_pool2_bwd(const bf16* __restrict__ dy, bf16* __restrict__ dx, int N, int H, int W, int C) {
  const long n = (long)N * H * W * C;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long q = i / C;
    const int xx = (int)(q % W), yy = (int)((q / W) % H);
    const long b = q / ((long)W * H);
    dx[i] = __float2bfloat16_rn(0.25f * __bfloat162float(dy[((b * (H / 2) + yy / 2) * (W / 2) + xx / 2) * C + c]));
  }
}

// y[n][y][x][c] = x[n][y/2][x/2][c] (H, W: the input's; the output is 2H x 2W).
__global__ void k_up2(const bf16* __restrict__ x, bf16* __restrict__ y, int N, int H, int W, int C) {
  const int Ho = 2 * H, Wo = 2 * W;
  const long n = (long)N * Ho * Wo * C;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long q = i / C;
    const int xx = (int)(q % Wo), yy = (int)((q / Wo) % Ho);
    const long b = q / ((long)Wo * Ho);
    y[i] = x[((b * H + yy / 2) * W + xx / 2) * C + c];
  }
}

// dx[n][i][j][c] = sum of dy over the 2x2 block (H, W: the upsampling's input).
__global__ void k_up2_bwd(const bf16* __restrict__ dy, bf16* __restrict__ dx, int N, int H, int W, int C) {
  const long n = (long)N * H * W * C;
  const int Wo = 2 * W;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long q = i / C;
    const int j = (int)(q % W), ii = (int)((q / W) % H);
    const long b = q / ((long)W * H);
    const long s = ((b * 2 * H + 2 * ii) * Wo + 2 * j) * C + c;
    const float v = __bfloat162float(dy[s]) + __bfloat162float(dy[s + C]) + __bfloat162float(dy[s + (long)Wo * C]) +
                    __bfloat162float(dy[s + (long)Wo * C + C]);
    dx[i] = __float2bfloat16_rn(v);
  }
}

__global__ void k_add(const bf16* __restrict__ a, const bf16* __restrict__ b, bf16* __restrict__ out, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(__bfloat162float(a[i]) + __bfloat162float(b[i]));
}

// Network input, 16 channels per pixel: (height - 0.25) * 4, the wind
// direction's x and z components, zeros.
__global__ void k_pack_input(const float* __restrict__ h, const float* __restrict__ wind_xz, bf16* __restrict__ x,
                             int N, int H, int W) {
  const long n = (long)N * H * W;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
    const long b = p / ((long)H * W);
    bf16* o = x + p * 16;
    o[0] = __float2bfloat16_rn((h[p] - 0.25f) * 4.0f);
    o[1] = __float2bfloat16_rn(wind_xz[2 * b]);
    o[2] = __float2bfloat16_rn(wind_xz[2 * b + 1]);
#pragma unroll
    for (int c = 3; c < 16; c++) o[c] = __float2bfloat16_rn(0.0f);
  }
}

// Squared-error loss on channel 0 of pred (C channels) against target *
// tscale: sum of squares into *loss, d pred = 2 (pred - target tscale)
// gscale on channel 0, zero elsewhere.
__global__ void k_mse(const bf16* __restrict__ pred, const float* __restrict__ target, float tscale,
                      bf16* __restrict__ dpred, float* __restrict__ loss, long M, int C, float scale) {
  float s = 0.0f;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < M; p += (long)gridDim.x * blockDim.x) {
    const float e = __bfloat162float(pred[p * C]) - target[p] * tscale;
    s += e * e;
    dpred[p * C] = __float2bfloat16_rn(2.0f * e * scale);
    for (int c = 1; c < C; c++) dpred[p * C + c] = __float2bfloat16_rn(0.0f);
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
  const long warps = ((M + 15) / 16) * ((cout + 8 * kConvNT - 1) / (8 * kConvNT));
  const long blocks = (warps * 32 + 127) / 128;
  k_conv3x3<<<(unsigned)blocks, 128, 0, s>>>(static_cast<const bf16*>(x), static_cast<const bf16*>(w), bias,
                                             static_cast<bf16*>(y), N, H, W, cin, cout);
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
  const long warps = ((M + kWgChunk - 1) / kWgChunk) * ((cout + 15) / 16) * ((9 * cin) / (8 * kWgNT));
  const long blocks = (warps * 32 + 127) / 128;
  k_conv_wgrad<<<(unsigned)blocks, 128, 0, s>>>(static_cast<const bf16*>(x), static_cast<const bf16*>(dy), dw, N, H,
                                                W, cin, cout);
  if (db) {
    long bx = (M + 255) / 256;
    if (bx > 64) bx = 64;
    k_bias_grad<<<dim3((unsigned)bx, (unsigned)cout), 256, 0, s>>>(static_cast<const bf16*>(dy), db, M, cout);
  }
  return cudaGetLastError();
}

cudaError_t nn_gelu(const void* pre, void* act, long n, cudaStream_t s) {
  k_gelu<<<grid_for(n), 256, 0, s>>>(static_cast<const bf16*>(pre), static_cast<bf16*>(act), n);
  return cudaGetLastError();
}

cudaError_t nn_gelu_bwd(const void* pre, const void* dact, void* dpre, long n, cudaStream_t s) {
  k_gelu_bwd<<<grid_for(n), 256, 0, s>>>(static_cast<const bf16*>(pre), static_cast<const bf16*>(dact),
                                         static_cast<bf16*>(dpre), n);
  return cudaGetLastError();
}

cudaError_t nn_pool2(const void* x, void* y, int N, int H, int W, int C, bool backward, cudaStream_t s) {
  const long n = (long)N * H * W * C;
  if (backward)
    k_pool2_bwd<<<grid_for(n), 256, 0, s>>>(static_cast<const bf16*>(x), static_cast<bf16*>(y), N, H, W, C);
  else
    k_pool2<<<grid_for(n / 4), 256, 0, s>>>(static_cast<const bf16*>(x), static_cast<bf16*>(y), N, H, W, C);
  return cudaGetLastError();
}

cudaError_t nn_up2(const void* x, void* y, int N, int H, int W, int C, bool backward, cudaStream_t s) {
  const long n = (long)N * H * W * C;
  if (backward)
    k_up2_bwd<<<grid_for(n), 256, 0, s>>>(static_cast<const bf16*>(x), static_cast<bf16*>(y), N, H, W, C);
  else
    k_up2<<<grid_for(4 * n), 256, 0, s>>>(static_cast<const bf16*>(x), static_cast<bf16*>(y), N, H, W, C);
  return cudaGetLastError();
}

cudaError_t nn_add(const void* a, const void* b, void* out, long n, cudaStream_t s) {
  k_add<<<grid_for(n), 256, 0, s>>>(static_cast<const bf16*>(a), static_cast<const bf16*>(b), static_cast<bf16*>(out),
                                    n);
  return cudaGetLastError();
}

cudaError_t nn_pack_input(const float* h, const float* wind_xz, void* x, int N, int H, int W, cudaStream_t s) {
  k_pack_input<<<grid_for((long)N * H * W), 256, 0, s>>>(h, wind_xz, static_cast<bf16*>(x), N, H, W);
  return cudaGetLastError();
}

cudaError_t nn_mse(const void* pred, const float* target, float tscale, void* dpred, float* loss, long M, int C,
                   float gscale, cudaStream_t s) {
  k_mse<<<grid_for(M), 256, 0, s>>>(static_cast<const bf16*>(pred), target, tscale, static_cast<bf16*>(dpred), loss,
                                    M, C, gscale);
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

}  // namespace

extern "C" {

int swe_nn_conv3x3(const void* x, const void* w, const float* bias, void* y, int n, int h, int wd, int cin, int cout,
                   void* stream) {
  if (!x || !w || !y) return nn_fail(SWE_ERR_INVALID, "NULL tensor");
  if (n < 1 || h < 1 || wd < 1 || cin < 16 || cin % 16 || cout < 8 || cout % 8)
    return nn_fail(SWE_ERR_INVALID, "conv3x3: need n, h, w >= 1, cin % 16 == 0, cout % 8 == 0");
  if (!aligned4(x) || !aligned4(w) || !aligned4(y)) return nn_fail(SWE_ERR_INVALID, "tensors must be 4-byte aligned");
  return nn_done(swe::nn_conv3x3(x, w, bias, y, n, h, wd, cin, cout, static_cast<cudaStream_t>(stream)));
}

int swe_nn_conv3x3_flip(const void* w, void* wf, int cin, int cout, void* stream) {
  if (!w || !wf || cin < 1 || cout < 1) return nn_fail(SWE_ERR_INVALID, "conv3x3_flip: bad arguments");
  return nn_done(swe::nn_flip(w, wf, cin, cout, static_cast<cudaStream_t>(stream)));
}

int swe_nn_conv3x3_wgrad(const void* x, const void* dy, float* dw, float* db, int n, int h, int wd, int cin, int cout,
                         void* stream) {
  if (!x || !dy || !dw) return nn_fail(SWE_ERR_INVALID, "NULL tensor");
  if (n < 1 || h < 1 || wd < 1 || cin < 16 || cin % 16 || cout < 8 || cout % 8)
    return nn_fail(SWE_ERR_INVALID, "conv3x3_wgrad: need n, h, w >= 1, cin % 16 == 0, cout % 8 == 0");
  return nn_done(swe::nn_conv_wgrad(x, dy, dw, db, n, h, wd, cin, cout, static_cast<cudaStream_t>(stream)));
}

int swe_nn_gelu(const void* pre, void* act, int64_t count, void* stream) {
  if (!pre || !act || count < 0) return nn_fail(SWE_ERR_INVALID, "gelu: bad arguments");
  if (count == 0) return SWE_OK;
  return nn_done(swe::nn_gelu(pre, act, (long)count, static_cast<cudaStream_t>(stream)));
}

int swe_nn_gelu_bwd(const void* pre, const void* dact, void* dpre, int64_t count, void* stream) {
  if (!pre || !dact || !dpre || count < 0) return nn_fail(SWE_ERR_INVALID, "gelu_bwd: bad arguments");
  if (count == 0) return SWE_OK;
  return nn_done(swe::nn_gelu_bwd(pre, dact, dpre, (long)count, static_cast<cudaStream_t>(stream)));
}

int swe_nn_pool2(const void* x, void* y, int n, int h, int wd, int c, int backward, void* stream) {
  if (!x || !y || n < 1 || h < 2 || wd < 2 || h % 2 || wd % 2 || c < 1)
    return nn_fail(SWE_ERR_INVALID, "pool2: need even h, w >= 2");
  return nn_done(swe::nn_pool2(x, y, n, h, wd, c, backward != 0, static_cast<cudaStream_t>(stream)));
}

int swe_nn_up2(const void* x, void* y, int n, int h, int wd, int c, int backward, void* stream) {
  if (!x || !y || n < 1 || h < 1 || wd < 1 || c < 1) return nn_fail(SWE_ERR_INVALID, "up2: bad arguments");
  return nn_done(swe::nn_up2(x, y, n, h, wd, c, backward != 0, static_cast<cudaStream_t>(stream)));
}

int swe_nn_add(const void* a, const void* b, void* out, int64_t count, void* stream) {
  if (!a || !b || !out || count < 0) return nn_fail(SWE_ERR_INVALID, "add: bad arguments");
  if (count == 0) return SWE_OK;
  return nn_done(swe::nn_add(a, b, out, (long)count, static_cast<cudaStream_t>(stream)));
}

int swe_nn_pack_input(const float* height, const float* wind_xz, void* x, int n, int h, int wd, void* stream) {
  if (!height || !wind_xz || !x || n < 1 || h < 1 || wd < 1) return nn_fail(SWE_ERR_INVALID, "pack_input: bad arguments");
  return nn_done(swe::nn_pack_input(height, wind_xz, x, n, h, wd, static_cast<cudaStream_t>(stream)));
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
