// Blackwell tensor-core convolutions of the learned surrogate (sm_103a):
// tcgen05.mma with the accumulators in tensor memory (TMEM), operand tiles
// brought into shared memory by the tensor-memory accelerator (TMA), and a
// multi-stage mbarrier pipeline.
//
//   k_conv_tc   3x3 convolution, zero padding, NHWC bf16, as an implicit
//               GEMM: rows = 128-pixel tiles of the output (taken two at a
//               time: a unit), columns = output channels, K = 9 taps x
//               input channels. Persistent: up to three CTAs per SM stride
//               over the units. The TMA loads the inputs straight from the
//               NHWC tensor (pixels beyond the map edge arrive as zeros: the
//               padding costs nothing) and the weight slices straight from
//               the [n][tap][k] weights, in one of two schemes: a unit of
//               two vertically adjacent tiles takes per k-block (dx, KC =
//               64, 32 or 16 input channels) one box of the dx-shifted input
//               covering its rows and one row above and below, which the
//               three dy taps read at offsets of whole image rows; a unit of
//               two consecutive tiles takes per k-block (tap, KC channels)
//               one tap-shifted box per tile. One
//               thread issues the copies, one the MMAs into one of two TMEM
//               accumulator sets; four warps run the epilogue of the other
//               set (TMEM -> registers, + bias, optional fused GELU, bf16
//               stores). The input gradient is the same kernel on the
//               output gradient with the weights flipped and transposed.
//               Its operands sit in shared memory in the canonical K-major
//               swizzled layout: one row of KC channels (128, 64 or 32
//               bytes) per pixel or output channel, 8-row atoms SBO = 8 rows
//               apart, the TMA writing the matching 128/64/32-byte swizzle;
//               full rows keep every L2 sector access whole.
//   k_wgrad_tc  the weight gradient: per tap a GEMM with M = output
//               channels, N = input channels, K = pixels, both operands
//               MN-major in the canonical swizzled layout: a TMA box of MA
//               channels x the tile's 128 pixels, the next MA channels one
//               box further on; one dy tile per k-block serves up to nine
//               tap-shifted x tiles. The bias gradient rides along (dy
//               against a block of ones in shared memory).
//
// Every wait on an mbarrier is bounded (2 s by the global timer): past it the
// kernel records an error code in g_tc_error, stops issuing work, waits
// (bounded) for the copies it already issued, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "swe_kernels.h"
#include "swe_nn_math.cuh"

namespace swe {
namespace {

using bf16 = __nv_bfloat16;

__device__ unsigned int g_tc_error;  // first failure code of a tensor-core kernel (0: none)

constexpr int kTcThreads = 128;
constexpr int kTcMTiles = 2;  // 128-pixel M tiles per unit of work (they share each weight slice)
constexpr unsigned long long kTcWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long tc_now() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the phase of `bar` with parity `parity`. Gives up when another
// role of the CTA has given up (*abort != 0, if `watch`) or after the
// deadline, recording `code`. Returns false if it gave up.
__device__ __noinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort, bool watch,
                                       unsigned code) {
  unsigned long long t0 = 0;
  for (uint32_t i = 0;; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 31u) == 31u) {
      if (watch && *abort) return false;
      const unsigned long long now = tc_now();
      if (t0 == 0) {
        t0 = now;
      } else if (now - t0 > kTcWaitNs) {
        atomicCAS(&g_tc_error, 0u, code);
        *abort = 1;
        return false;
      }
    }
  }
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// The same for a K-major operand in a swizzled layout (layout code `swz` in
// bits 61-63: 2 = 128-byte, 4 = 64-byte, 6 = 32-byte swizzle): rows of one
// swizzle span, 8-row atoms SBO bytes apart; LBO is not used (encoded 1).
// Moving along K within a row adds the byte offset to the start address.
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t addr, uint32_t sbo, uint32_t swz) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) |
         ((uint64_t)swz << 61);
}

// General form: start address, LBO, SBO, layout code (0 = no swizzle).
__device__ __forceinline__ uint64_t smem_desc_full(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t swz) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46) | ((uint64_t)swz << 61);
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

// Instruction descriptor of kind::f16: bf16 A and B, fp32 D, both K-major,
// M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// The same with both operands MN-major (the M or N index contiguous):
// transpose bits 15 (A) and 16 (B).
__host__ __device__ constexpr uint32_t idesc_bf16_mn(int m, int n) { return idesc_bf16(m, n) | (1u << 15) | (1u << 16); }

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives on `bar` once every MMA this thread issued before has completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}


__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi)) << 16);
}

struct TcConvGeom {
  int H, W;
  int kc;      // GEMM K channels (input channels of this convolution)
  int nc;      // GEMM N (output channels)
  int TW, R;   // an M tile: R image rows x TW pixels = 128 pixels
  int KC;      // channels per k-block: 64, 32 or 16, one swizzled row of 128, 64 or 32 bytes per pixel
  int chunks;  // kc / KC
  int vertical;  // 1: a unit is kTcMTiles vertically adjacent tiles and a k-block (dx, chunk) takes one
                 // input box of the unit's rows and one row above and below, which serves the three dy
                 // taps; 0: a unit is kTcMTiles consecutive tiles and a k-block (tap, chunk) takes one
                 // tap-shifted box per tile
  int tpr;       // tiles side by side in a row group (W / TW)
  int rgroups;   // row groups of R image rows in a map (H / R)
  int ublocks;   // vertical units stacked in a column of tiles (rgroups / kTcMTiles, rounded up)
  int tiles;     // 128-pixel tiles in the batch
  int units;     // units of work
  int xrows;     // image rows of one input box: R kTcMTiles + 2 (vertical) or R
  int x_bytes;   // bytes of the input boxes per k-block (kTcMTiles x 128 or xrows x TW rows of KC channels)
  int col_stride;  // TMEM columns between the M tiles of a unit
  int nbuf;        // TMEM accumulator sets (2: the epilogue of one unit overlaps the next unit's MMAs)
  int ncols;       // TMEM columns allocated
  int b_bytes;     // bytes of one tap's weight slice (nc rows of KC channels); three per k-block if vertical
  int stage_bytes;
  int stages;      // pipeline depth (2..6)
  uint32_t swz;    // descriptor layout code of the swizzle
};

// warp 0 copies, warp 1 issues the MMAs, warps 2-5 run the epilogue (warp w
// may read TMEM lanes 32 (w % 4) .. + 31). Up to three CTAs share an SM
// (each its own copy/MMA pipeline): with one CTA per SM the copies of a
// tile's nine tap-shifted boxes, issued one after another by one thread,
// set the pace.
constexpr int kConvWarps = 6;

// Tile mt of unit u: its image n and top-left pixel (y, x); returns the
// unit's tile count.
__device__ __forceinline__ int unit_tile(const TcConvGeom& g, int u, int mt, int& n, int& y, int& x) {
  if (g.vertical) {
    const int upi = g.tpr * g.ublocks, q = u % upi, rg0 = (q / g.tpr) * kTcMTiles;
    n = u / upi;
    x = (q % g.tpr) * g.TW;
    y = (rg0 + mt) * g.R;
    return min(kTcMTiles, g.rgroups - rg0);
  }
  const int t = u * kTcMTiles + mt, tpi = g.tpr * g.rgroups, q = t % tpi;
  n = t / tpi;
  y = (q / g.tpr) * g.R;
  x = (q % g.tpr) * g.TW;
  return min(kTcMTiles, g.tiles - u * kTcMTiles);
}
constexpr int kConvEpilogueWarps = kConvWarps - 2;
constexpr int kConvMaxCtasPerSm = 3;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Persistent: each CTA takes units (two M tiles each) blockIdx.x,
// blockIdx.x + gridDim.x, ...; the copies and MMAs run ahead through the
// units' k-blocks in one stage ring while the epilogue warps drain the
// previous unit's accumulators from the other TMEM set.
__global__ void __launch_bounds__(kConvWarps * 32, kConvMaxCtasPerSm)
    k_conv_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap wmap,
              const float* __restrict__ bias, bf16* __restrict__ y, bf16* __restrict__ act, const TcConvGeom g) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + g.stages * g.stage_bytes);
  uint64_t* empty = full + 8;
  uint64_t* tfull = empty + 8;   // accumulator set b holds a finished unit
  uint64_t* tempty = tfull + 2;  // accumulator set b was drained by the epilogue
  uint64_t* drain = tempty + 2;  // every MMA this CTA issued has completed
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* consumed = abort + 1;  // k-blocks whose data the MMA thread took

  __shared__ __align__(16) float s_bias[256];  // the bias (zeros without one), read by the epilogue
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kblocks = (g.vertical ? 3 : 9) * g.chunks;  // (dx, chunk) or (tap, chunk)
  const int ntap = g.vertical ? 3 : 1;                   // taps per k-block
  for (int i = threadIdx.x; i < g.nc; i += blockDim.x) s_bias[i] = bias ? bias[i] : 0.0f;

  if (threadIdx.x == 0) {
    for (int s = 0; s < g.stages; s++) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(tfull + b, 1);
      mbar_init(tempty + b, kConvEpilogueWarps);
    }
    mbar_init(drain, 1);
    *abort = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(g.ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int issued = 0;  // producer: k-blocks whose copies were issued
  if (warp == 0) {
    if (lane == 0) {
      // ---- producer: per k-block (vertical) one box of the dx-shifted input
      // covering the unit's rows and one row above and below and the three
      // dy taps' weight slices, or (otherwise) one tap-shifted box per tile
      // and the tap's weight slice; pixels past the map edge arrive as zeros
      int kbg = 0;
      for (int u = blockIdx.x; u < g.units && !*abort; u += gridDim.x) {
        int tn[kTcMTiles], ty[kTcMTiles], tx[kTcMTiles];
        int mt_n = 0;
#pragma unroll
        for (int mt = 0; mt < kTcMTiles; mt++) mt_n = unit_tile(g, u, mt, tn[mt], ty[mt], tx[mt]);
        const uint32_t bytes = g.vertical ? (uint32_t)g.x_bytes + 3u * (uint32_t)g.b_bytes
                                          : (uint32_t)(mt_n * 128 * 2 * g.KC + g.b_bytes);
        bool ok = true;
        for (int kb = 0; kb < kblocks; kb++, kbg++) {
          const int s = kbg % g.stages;
          const uint32_t ph = (uint32_t)(kbg / g.stages) & 1u;
          if (!mbar_wait(empty + s, ph ^ 1u, abort, true, 1u)) {
            ok = false;
            break;
          }
          const int kq = kb / g.chunks, chunk = kb % g.chunks;  // kq: dx + 1 (vertical) or the tap
          unsigned char* st = smem + s * g.stage_bytes;
          mbar_expect_tx(full + s, bytes);
          if (g.vertical) {
            tma_load_4d(st, &xmap, full + s, chunk * g.KC, tx[0] + kq - 1, ty[0] - 1, tn[0]);
            for (int dy = 0; dy < 3; dy++)
              tma_load_3d(st + g.x_bytes + dy * g.b_bytes, &wmap, full + s, chunk * g.KC, dy * 3 + kq, 0);
          } else {
            const int dy = kq / 3 - 1, dx = kq % 3 - 1;
            for (int mt = 0; mt < mt_n; mt++)
              tma_load_4d(st + mt * 128 * 2 * g.KC, &xmap, full + s, chunk * g.KC, tx[mt] + dx, ty[mt] + dy, tn[mt]);
            tma_load_3d(st + g.x_bytes, &wmap, full + s, chunk * g.KC, kq, 0);
          }
          issued = kbg + 1;
        }
        if (!ok) break;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer
      const uint32_t idesc = idesc_bf16(128, g.nc);
      const uint32_t sb = smem_u32(smem);
      const uint32_t sbo = 16u * (uint32_t)g.KC;  // 8 rows of KC bf16
      int kbg = 0, it = 0;
      bool ok = true;
      const uint32_t row_bytes = 2u * (uint32_t)g.KC;
      for (int u = blockIdx.x; u < g.units && ok; u += gridDim.x, it++) {
        int n0, y0, x0;
        const int mt_n = unit_tile(g, u, 0, n0, y0, x0);
        const int b = it % g.nbuf, use = it / g.nbuf;
        if (!mbar_wait(tempty + b, (uint32_t)(use & 1) ^ 1u, abort, true, 5u)) break;
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(b * kTcMTiles * g.col_stride);
        for (int kb = 0; kb < kblocks; kb++, kbg++) {
          const int s = kbg % g.stages;
          const uint32_t ph = (uint32_t)(kbg / g.stages) & 1u;
          if (!mbar_wait(full + s, ph, abort, true, 2u)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t x_base = sb + s * g.stage_bytes, w_base = x_base + g.x_bytes;
          for (int mt = 0; mt < mt_n; mt++) {
            for (int dy = 0; dy < ntap; dy++) {
              // tile mt's 128 pixels (shifted by dy rows if vertical): box rows
              // (mt R + dy) TW on, a whole number of 8-row swizzle atoms (TW >= 8)
              const uint32_t a0 = x_base + (uint32_t)((mt * g.R + dy) * g.TW) * row_bytes;
              const uint32_t b0 = w_base + (uint32_t)(dy * g.b_bytes);
              for (int j = 0; j < g.KC / 16; j++) {
                const uint64_t ad = smem_desc_sw(a0 + 32 * j, sbo, g.swz);
                const uint64_t bd = smem_desc_sw(b0 + 32 * j, sbo, g.swz);
                umma_bf16(acc + mt * g.col_stride, ad, bd, idesc, (kb > 0 || dy > 0 || j > 0) ? 1u : 0u);
              }
            }
          }
          umma_commit(empty + s);  // the stage is free once these MMAs have read it
        }
        umma_commit(tfull + b);  // the unit's accumulators are complete (or the unit was cut short)
      }
      *consumed = kbg;
      umma_commit(drain);
      mbar_wait(drain, 0u, abort, false, 6u);
    }
  } else {
    // ---- epilogue: warps 2-5; warp w reads TMEM lanes 32 (w % 4) .. + 31
    // (with more epilogue warps, kPerQuarter share a quarter's chunks)
    const int q4 = warp & 3, l = q4 * 32 + lane, half = (warp - 2) >> 2;
    constexpr int kPerQuarter = kConvEpilogueWarps / 4;  // warps per TMEM lane quarter
    int it = 0;
    for (int u = blockIdx.x; u < g.units; u += gridDim.x, it++) {
      int img0, row00, col00;
      const int mt_n = unit_tile(g, u, 0, img0, row00, col00);
      const int b = it % g.nbuf, use = it / g.nbuf;
      const bool have = mbar_wait(tfull + b, (uint32_t)(use & 1), abort, true, 3u);
      tc_fence_after();
      if (!__all_sync(0xffffffffu, have && *abort == 0)) break;
      const uint32_t acc = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(b * kTcMTiles * g.col_stride);
      for (int mt = 0; mt < mt_n; mt++) {
        // TMEM lane l of tile mt is image pixel (row0 + l / TW, col0 + l % TW)
        // (names that do not hide the output pointer y)
        int img, row0, col0;
        unit_tile(g, u, mt, img, row0, col0);
        const long pix = ((long)img * g.H + row0 + l / g.TW) * g.W + col0 + l % g.TW;
        for (int j = half; j < g.nc / 16; j += kPerQuarter) {
          float v[16];
          tmem_ld16(acc + mt * g.col_stride + 16 * j, v);
          const float4* bq = reinterpret_cast<const float4*>(s_bias + 16 * j);
#pragma unroll
          for (int i = 0; i < 4; i++) {
            const float4 b4 = bq[i];
            v[4 * i] += b4.x;
            v[4 * i + 1] += b4.y;
            v[4 * i + 2] += b4.z;
            v[4 * i + 3] += b4.w;
          }
          uint32_t w[8];
#pragma unroll
          for (int i = 0; i < 8; i++) w[i] = pack_bf16(v[2 * i], v[2 * i + 1]);
          uint4* dst = reinterpret_cast<uint4*>(y + pix * g.nc + 16 * j);
          dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
          dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
          if (act) {
            // GELU of the bf16-rounded pre-activation (the values just
            // packed), as the separate GELU pass computes it
            uint32_t a[8];
#pragma unroll
            for (int i = 0; i < 8; i++)
              a[i] = pack_bf16(gelu_as(__uint_as_float(w[i] << 16)), gelu_as(__uint_as_float(w[i] & 0xFFFF0000u)));
            uint4* da = reinterpret_cast<uint4*>(act + pix * g.nc + 16 * j);
            da[0] = make_uint4(a[0], a[1], a[2], a[3]);
            da[1] = make_uint4(a[4], a[5], a[6], a[7]);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(tempty + b);  // this warp is done with set b
    }
  }

  // ---- teardown: no copy may land after the CTA exits, and TMEM is freed
  __syncthreads();  // the MMA thread's count of consumed k-blocks is visible
  if (warp == 0 && lane == 0) {
    for (int kb = *consumed; kb < issued; kb++)
      mbar_wait(full + kb % g.stages, (uint32_t)(kb / g.stages) & 1u, abort, false, 4u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.ncols) : "memory");
}

struct TcWgradGeom {
  int H, W, cin, cout;
  int TW, R;          // a pixel tile: R image rows x TW pixels = 128 pixels
  int MA, MB;         // channels per swizzled row of dy (A) and of x (B): 64, 32 or 16
  uint32_t swzA, swzB;
  int tiles;          // 128-pixel tiles in the batch
  int tiles_per_cta;  // the CTA's share of the pixel sum (split K)
  int taps;           // taps per CTA (9, or 3: one row of taps per blockIdx.y)
  int kt;             // taps per k-block: one dy tile serves kt tap-shifted x tiles (kt divides taps)
  int col_stride;     // TMEM columns per tap
  int ncols;
  int stages;
  int a_bytes, stage_bytes;
  int tail;  // bytes after the stages, so that the padded M rows of the last A operand stay in the allocation
  int db_col;  // TMEM column of the bias-gradient accumulator (CTAs of tap group 0, with db), or -1
};

// Weight gradient dW[co][tap][ci] += sum over pixels p of dy[p][co] x[p + tap][ci]
// as a GEMM per tap with M = output channels (padded to 128; the rows past
// cout are never stored), N = input channels, K = pixels, split over CTAs by
// pixel tiles and over blockIdx.y by rows of taps. Both operands are
// MN-major (channels contiguous) in the canonical swizzled layout: a TMA box
// of MA (or MB) channels x the tile's 128 pixels is 128 rows of MA*2 bytes
// along K (8-row atoms SBO = 16*MA bytes apart; a 16-pixel K step is two of
// them), the next MA channels one box further on (LBO = 256*MA bytes along M
// or N). Per k-block (one 128-pixel tile, kt taps) the TMA brings the dy
// tile once and the kt tap-shifted x tiles (zeros past the map edge). The
// partial sums leave TMEM through fp32 atomics into dw.
__global__ void __launch_bounds__(kTcThreads, 1)
    k_wgrad_tc(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap dymap,
               float* __restrict__ dw, float* __restrict__ db, const TcWgradGeom g) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  // 16 channels x 128 pixels of bf16 ones (4 KiB, after the stages and the
  // tail): the B operand of the bias gradient, db[co] = sum_p dy[p][co] x 1
  unsigned char* ones = smem + (g.stages * g.stage_bytes + g.tail + 1023) / 1024 * 1024;
  uint64_t* full = reinterpret_cast<uint64_t*>(ones + 4096);
  uint64_t* empty = full + 4;
  uint64_t* accum = empty + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accum + 1);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* consumed = abort + 1;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t0 = blockIdx.x * g.tiles_per_cta;
  const int nt = max(0, min(g.tiles_per_cta, g.tiles - t0));
  const int tap0 = blockIdx.y * g.taps;
  const int gk = g.taps / g.kt;  // k-blocks per tile
  const int kblocks = nt * gk;
  const bool with_db = db != nullptr && blockIdx.y == 0 && g.db_col >= 0;
  if (with_db) {
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) reinterpret_cast<uint32_t*>(ones)[i] = 0x3F803F80u;
    // the MMAs read it through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }

  if (threadIdx.x == 0) {
    for (int s = 0; s < g.stages; s++) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    mbar_init(accum, 1);
    *abort = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(g.ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int issued = 0;
  if (warp == 0 && lane == 0) {
    const int tiles_per_img = (g.H * g.W) >> 7;
    // 8 K steps x 16 pixels x channels x 2 bytes: the dy tile and kt x tiles
    const uint32_t bytes = 256u * (uint32_t)(g.cout + g.kt * g.cin);
    for (int kb = 0; kb < kblocks; kb++) {
      const int s = kb % g.stages;
      const uint32_t ph = (uint32_t)(kb / g.stages) & 1u;
      if (!mbar_wait(empty + s, ph ^ 1u, abort, true, 11u)) break;
      const int t = t0 + kb / gk, tapk = tap0 + (kb % gk) * g.kt;
      const int q = t % tiles_per_img, tn = t / tiles_per_img;
      const int ty = (q / (g.W / g.TW)) * g.R, tx = (q % (g.W / g.TW)) * g.TW;
      unsigned char* st = smem + s * g.stage_bytes;
      mbar_expect_tx(full + s, bytes);
      // one box per MA (MB) channels: the tile's 128 pixels as 128 rows
      for (int m = 0; m < g.cout / g.MA; m++)
        tma_load_4d(st + m * 256 * g.MA, &dymap, full + s, m * g.MA, tx, ty, tn);
      for (int k = 0; k < g.kt; k++) {
        const int dy = (tapk + k) / 3 - 1, dx = (tapk + k) % 3 - 1;
        unsigned char* xs = st + g.a_bytes + k * 256 * g.cin;
        for (int m = 0; m < g.cin / g.MB; m++)
          tma_load_4d(xs + m * 256 * g.MB, &xmap, full + s, m * g.MB, tx + dx, ty + dy, tn);
      }
      issued = kb + 1;
    }
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = idesc_bf16_mn(128, g.cin);
    const uint32_t idesc16 = idesc_bf16_mn(128, 16);
    const uint32_t sb = smem_u32(smem), so = smem_u32(ones);
    int kb = 0;
    for (; kb < kblocks; kb++) {
      const int s = kb % g.stages;
      const uint32_t ph = (uint32_t)(kb / g.stages) & 1u;
      if (!mbar_wait(full + s, ph, abort, true, 12u)) break;
      tc_fence_after();
      const int i = kb / gk, j0 = (kb % gk) * g.kt;
      const uint32_t a0 = sb + s * g.stage_bytes;
      for (int k = 0; k < g.kt; k++) {
        const uint32_t b0 = a0 + g.a_bytes + k * 256 * g.cin;
#pragma unroll
        for (int k16 = 0; k16 < 8; k16++) {
          const uint64_t ad = smem_desc_full(a0 + k16 * 32 * g.MA, 256 * g.MA, 16 * g.MA, g.swzA);
          const uint64_t bd = smem_desc_full(b0 + k16 * 32 * g.MB, 256 * g.MB, 16 * g.MB, g.swzB);
          umma_bf16(tmem + (j0 + k) * g.col_stride, ad, bd, idesc, (i > 0 || k16 > 0) ? 1u : 0u);
        }
      }
      if (with_db && j0 == 0) {
        // once per pixel tile: dy against the ones (N = 16 identical columns)
#pragma unroll
        for (int k16 = 0; k16 < 8; k16++) {
          const uint64_t ad = smem_desc_full(a0 + k16 * 32 * g.MA, 256 * g.MA, 16 * g.MA, g.swzA);
          const uint64_t od = smem_desc_full(so + k16 * 32 * 16, 256 * 16, 16 * 16, 6u);
          umma_bf16(tmem + (uint32_t)g.db_col, ad, od, idesc16, (i > 0 || k16 > 0) ? 1u : 0u);
        }
      }
      umma_commit(empty + s);
    }
    *consumed = kb;
    umma_commit(accum);
  }

  __syncwarp();
  const bool have = mbar_wait(accum, 0u, abort, false, 13u);
  tc_fence_after();
  if (__all_sync(0xffffffffu, have && *abort == 0) && nt > 0) {
    const int co = warp * 32 + lane;  // TMEM lane = output channel
    for (int j = 0; j < g.taps; j++) {
      for (int c16 = 0; c16 < g.cin / 16; c16++) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + j * g.col_stride + 16 * c16, v);
        if (co < g.cout) {
          float* dst = dw + ((long)co * 9 + tap0 + j) * g.cin + 16 * c16;
#pragma unroll
          for (int i = 0; i < 16; i++) atomicAdd(dst + i, v[i]);
        }
      }
    }
    if (with_db) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)g.db_col, v);
      if (co < g.cout) atomicAdd(db + co, v[0]);
    }
  }

  __syncthreads();
  if (warp == 0 && lane == 0) {
    for (int kb = *consumed; kb < issued; kb++)
      mbar_wait(full + kb % g.stages, (uint32_t)(kb / g.stages) & 1u, abort, false, 14u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.ncols) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

}  // namespace

// Width of a 128-pixel M tile: the largest power of two up to 128 dividing
// the map width (a tile is 128 / TW rows of TW pixels).
static int tile_width(int W) {
  int tw = 128;
  while (tw > 1 && W % tw != 0) tw >>= 1;
  return tw;
}

bool nn_conv_tc_supported(int H, int W, int kc, int nc) {
  if (kc < 16 || kc % 16 != 0 || nc < 16 || nc % 16 != 0 || nc > 256) return false;
  const int TW = tile_width(W);
  return TW >= 8 && H % (128 / TW) == 0;
}

cudaError_t nn_pack_tc(const void* w, void* wp, int cin, int cout, bool flip, cudaStream_t s) {
  // The kernel reads weights as [n][tap][k] through a tensor map: the
  // forward weights as they are ([cout][3][3][cin]), the input gradient's
  // flipped and transposed ([cin][3][3][cout], tap -> 8 - tap).
  if (flip) return nn_flip(w, wp, cin, cout, s);
  return cudaMemcpyAsync(wp, w, sizeof(bf16) * 9 * (size_t)cin * cout, cudaMemcpyDeviceToDevice, s);
}

namespace {

// A bf16 tensor map over `rank` dims (innermost first) with the given box and
// the swizzle that matches a box row of `row_bytes` (128, 64 or 32).
cudaError_t make_map(CUtensorMap* map, const void* t, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
                     const cuuint32_t* box, int row_bytes) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  // every box fits inside its tensor (no dimension of a box exceeds the tensor's)
  for (int i = 0; i < rank; i++)
    if ((cuuint64_t)box[i] > dims[i]) return cudaErrorInvalidValue;
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUtensorMapSwizzle sw = row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                : row_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                  : CU_TENSOR_MAP_SWIZZLE_32B;
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(t), dims, strides,
                         box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

cudaError_t nn_conv_tc(const void* x, const void* wp, const float* bias, void* y, void* act, int N, int H, int W,
                       int kc, int nc, cudaStream_t s) {
  if (!nn_conv_tc_supported(H, W, kc, nc)) return cudaErrorNotSupported;
  if ((reinterpret_cast<uintptr_t>(x) & 15) || (reinterpret_cast<uintptr_t>(wp) & 15) ||
      (reinterpret_cast<uintptr_t>(y) & 15) || (act && (reinterpret_cast<uintptr_t>(act) & 15)))
    return cudaErrorMisalignedAddress;
  TcConvGeom g;
  g.H = H;
  g.W = W;
  g.kc = kc;
  g.nc = nc;
  g.TW = tile_width(W);
  g.R = 128 / g.TW;
  g.KC = kc % 64 == 0 ? 64 : (kc % 32 == 0 ? 32 : 16);
  g.chunks = kc / g.KC;
  g.tpr = W / g.TW;
  g.rgroups = H / g.R;
  g.ublocks = (g.rgroups + kTcMTiles - 1) / kTcMTiles;
  const long tiles = (long)N * g.tpr * g.rgroups;
  const long vunits = (long)N * g.tpr * g.ublocks;
  if (vunits > 0x7FFFFFFFl || tiles > 0x7FFFFFFFl) return cudaErrorNotSupported;
  g.tiles = (int)tiles;
  g.col_stride = 32;  // a power of two: every accumulator starts on a multiple of its width
  while (g.col_stride < nc) g.col_stride <<= 1;
  g.b_bytes = nc * g.KC * 2;
  g.swz = g.KC == 64 ? 2u : (g.KC == 32 ? 4u : 6u);
  // The unit scheme and the launch shape. For each scheme: the most CTAs
  // per SM (up to three), then two TMEM accumulator sets rather than one,
  // whose TMEM allocations fit in the SM's 512 columns and whose stage rings
  // (at least two stages each) fit in its 228 KiB of shared memory (less
  // 2 KiB per CTA for the static bias array and the system's reservation).
  // Then the scheme that copies fewer rows per unit and CTA: a unit's input
  // rows, one per pixel and k-block, are what sets the pace.
  struct Plan {
    int cps = 0, nbuf = 0, ncols = 0, stages = 0, x_bytes = 0, stage_bytes = 0;
    double cost = 0.0;
  };
  auto plan_for = [&](int vertical) {
    Plan p;
    const int xrows = vertical ? g.R * kTcMTiles + 2 : g.R;
    p.x_bytes = vertical ? xrows * g.TW * g.KC * 2 : kTcMTiles * 128 * g.KC * 2;
    p.stage_bytes = (p.x_bytes + (vertical ? 3 : 1) * g.b_bytes + 1023) / 1024 * 1024;
    for (int c = kConvMaxCtasPerSm; c >= 1 && !p.cps; c--) {
      const size_t budget = (size_t)228 * 1024 / c - 2048;
      int st = 6;
      while (st > 2 && 1024 + (size_t)st * p.stage_bytes + 256 > budget) st--;
      if (1024 + (size_t)st * p.stage_bytes + 256 > budget) continue;
      for (int nb = 2; nb >= 1 && !p.cps; nb--) {
        int cols = 32;
        while (cols < nb * kTcMTiles * g.col_stride) cols <<= 1;
        if (cols > 512 || c * cols > 512) continue;
        p.cps = c;
        p.nbuf = nb;
        p.ncols = cols;
        p.stages = st;
      }
    }
    const double rows = vertical ? 3.0 * xrows * g.TW : 9.0 * kTcMTiles * 128;
    p.cost = p.cps ? rows / p.cps : 1e30;
    return p;
  };
  // the vertical scheme's input box (R kTcMTiles + 2 rows) must fit in the map's height
  const Plan pv = g.R * kTcMTiles + 2 <= H ? plan_for(1) : Plan(), ph = plan_for(0);
  if (!pv.cps && !ph.cps) return cudaErrorNotSupported;
  g.vertical = pv.cps && (!ph.cps || pv.cost <= ph.cost) ? 1 : 0;
  const Plan& pl = g.vertical ? pv : ph;
  const int cps = pl.cps;
  g.nbuf = pl.nbuf;
  g.ncols = pl.ncols;
  g.stages = pl.stages;
  g.x_bytes = pl.x_bytes;
  g.stage_bytes = pl.stage_bytes;
  g.xrows = g.vertical ? g.R * kTcMTiles + 2 : g.R;
  g.units = g.vertical ? (int)vunits : (int)((tiles + kTcMTiles - 1) / kTcMTiles);
  size_t smem = 1024 + (size_t)g.stages * g.stage_bytes + 256;
  // at most cps CTAs on an SM (each holds TMEM): more than 1/(cps+1) of its shared memory each
  const size_t floor_smem = (size_t)228 * 1024 / (cps + 1) + 1;
  if (smem < floor_smem) smem = floor_smem;
  if (smem > 227 * 1024) return cudaErrorNotSupported;

  CUtensorMap xm, wm;
  const cuuint64_t xd[4] = {(cuuint64_t)kc, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
  const cuuint64_t xs[3] = {(cuuint64_t)kc * 2, (cuuint64_t)W * kc * 2, (cuuint64_t)H * W * kc * 2};
  const cuuint32_t xb[4] = {(cuuint32_t)g.KC, (cuuint32_t)g.TW, (cuuint32_t)g.xrows, 1};
  const cuuint64_t wd[3] = {(cuuint64_t)kc, 9, (cuuint64_t)nc};
  const cuuint64_t ws[2] = {(cuuint64_t)kc * 2, (cuuint64_t)9 * kc * 2};
  const cuuint32_t wb[3] = {(cuuint32_t)g.KC, 1, (cuuint32_t)nc};
  cudaError_t e = make_map(&xm, x, 4, xd, xs, xb, g.KC * 2);
  if (e == cudaSuccess) e = make_map(&wm, wp, 3, wd, ws, wb, g.KC * 2);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int slots = cps * (sms > 0 ? sms : 1);
  const int grid = g.units < slots ? g.units : slots;
  k_conv_tc<<<grid, kConvWarps * 32, smem, s>>>(xm, wm, bias, static_cast<bf16*>(y), static_cast<bf16*>(act), g);
  return cudaGetLastError();
}

bool nn_wgrad_tc_supported(int H, int W, int cin, int cout) {
  return nn_conv_tc_supported(H, W, cin, cin) && cout >= 16 && cout % 16 == 0 && cout <= 128 && cin <= 128;
}

cudaError_t nn_wgrad_tc(const void* x, const void* dy, float* dw, float* db, int N, int H, int W, int cin, int cout,
                        int sms, cudaStream_t s) {
  if (!nn_wgrad_tc_supported(H, W, cin, cout)) return cudaErrorNotSupported;
  if ((reinterpret_cast<uintptr_t>(x) & 15) || (reinterpret_cast<uintptr_t>(dy) & 15)) return cudaErrorMisalignedAddress;
  TcWgradGeom g;
  g.H = H;
  g.W = W;
  g.cin = cin;
  g.cout = cout;
  g.TW = tile_width(W);
  g.R = 128 / g.TW;
  g.MA = cout % 64 == 0 ? 64 : (cout % 32 == 0 ? 32 : 16);
  g.MB = cin % 64 == 0 ? 64 : (cin % 32 == 0 ? 32 : 16);
  g.swzA = g.MA == 64 ? 2u : (g.MA == 32 ? 4u : 6u);
  g.swzB = g.MB == 64 ? 2u : (g.MB == 32 ? 4u : 6u);
  g.tiles = (int)((long)N * H * W / 128);
  g.col_stride = (cin + 31) / 32 * 32;
  g.a_bytes = 256 * cout;  // 8 K steps x 16 pixels x cout x 2 bytes
  auto stage_of = [&](int kt) { return g.a_bytes + 256 * kt * cin; };
  // the MMA reads 128 rows of A (128 / MA blocks of 256 MA bytes = 32 KiB from
  // the stage's start): keep the last stage's reads inside the allocation
  auto tail_of = [&](int kt) { return stage_of(kt) < 32768 ? 32768 - stage_of(kt) : 0; };
  // The shape, in order of preference: the most CTAs per SM (up to three,
  // each its own copy/MMA pipeline), then the most taps per CTA (9 or 3:
  // TMEM columns), then the most taps per k-block (9, 3 or 1: one dy tile for
  // kt x tiles), with at least two stages in the CTA's share of the SM's
  // 228 KiB of shared memory.
  // with db, 32 more TMEM columns (the bias gradient's accumulator); the
  // 4 KiB block of ones (aligned to 1 KiB) always sits before the barriers
  const int db_cols = db ? 32 : 0;
  const size_t extra = 1024 + 4096;
  int cps = 0;
  for (int c = 3; c >= 1 && !cps; c--) {
    const size_t budget = (size_t)228 * 1024 / c - 1024;
    for (int taps = 9; taps >= 3 && !cps; taps /= 3) {
      if (taps * g.col_stride + db_cols > 512) continue;
      int cols = 32;
      while (cols < taps * g.col_stride + db_cols) cols <<= 1;
      if (c * cols > 512) continue;
      for (int kt = taps; kt >= 1 && !cps; kt /= 3) {
        int st = 4;
        while (st > 2 && 1024 + (size_t)st * stage_of(kt) + tail_of(kt) + extra + 128 > budget) st--;
        if (1024 + (size_t)st * stage_of(kt) + tail_of(kt) + extra + 128 > budget) continue;
        cps = c;
        g.taps = taps;
        g.ncols = cols;
        g.kt = kt;
        g.stages = st;
      }
    }
  }
  if (!cps) return cudaErrorNotSupported;
  g.stage_bytes = stage_of(g.kt);
  g.tail = tail_of(g.kt);
  g.db_col = db ? g.taps * g.col_stride : -1;
  // the ones start at the next 1 KiB after the stages and the tail; the barriers 4 KiB later
  size_t smem = 1024 + ((size_t)g.stages * g.stage_bytes + g.tail + 1023) / 1024 * 1024 + 4096 + 128;
  // at most cps CTAs on an SM (each holds TMEM): more than 1/(cps+1) of its shared memory each
  const size_t floor_smem = (size_t)228 * 1024 / (cps + 1) + 1;
  if (smem < floor_smem) smem = floor_smem;
  if (smem > 227 * 1024) return cudaErrorNotSupported;
  // one wave: cps CTAs per SM in all, each summing a run of pixel tiles
  const int groups = 9 / g.taps;
  int ctas_x = (cps * (sms > 0 ? sms : 148)) / groups;
  if (ctas_x < 1) ctas_x = 1;
  if (ctas_x > g.tiles) ctas_x = g.tiles;
  g.tiles_per_cta = (g.tiles + ctas_x - 1) / ctas_x;
  ctas_x = (g.tiles + g.tiles_per_cta - 1) / g.tiles_per_cta;
  CUtensorMap xm, dm;
  const cuuint64_t xd[4] = {(cuuint64_t)cin, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
  const cuuint64_t xs[3] = {(cuuint64_t)cin * 2, (cuuint64_t)W * cin * 2, (cuuint64_t)H * W * cin * 2};
  const cuuint32_t xb[4] = {(cuuint32_t)g.MB, (cuuint32_t)g.TW, (cuuint32_t)g.R, 1};
  const cuuint64_t dd[4] = {(cuuint64_t)cout, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
  const cuuint64_t ds[3] = {(cuuint64_t)cout * 2, (cuuint64_t)W * cout * 2, (cuuint64_t)H * W * cout * 2};
  const cuuint32_t dyb[4] = {(cuuint32_t)g.MA, (cuuint32_t)g.TW, (cuuint32_t)g.R, 1};
  cudaError_t e = make_map(&xm, x, 4, xd, xs, xb, g.MB * 2);
  if (e == cudaSuccess) e = make_map(&dm, dy, 4, dd, ds, dyb, g.MA * 2);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_wgrad_tc<<<dim3(ctas_x, groups), kTcThreads, smem, s>>>(xm, dm, dw, db, g);
  return cudaGetLastError();
}

cudaError_t nn_tc_status(unsigned int* code) {
  unsigned int v = 0;
  cudaError_t e = cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(v));
  if (e == cudaSuccess && v) {
    const unsigned int zero = 0;
    e = cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(zero));
  }
  *code = v;
  return e;
}

}  // namespace swe
