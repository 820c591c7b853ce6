// Parallel fixed-point erosion: all particles of an erode cycle fly together.
//
// One cycle (the World::erode(P) call, world.hpp:36-77) is
//   k_par_spawn                 zero the track accumulators, spawn P particles
//   (k_par_fly, 4 x k_par_cascade) x (max_age + 2) steps
//   k_par_ema                   tracks -> float, EMA of massflow/momentum
//                               (world.hpp:70-76), fixed-point heights -> float
//
// Step semantics.
//  fly      every live particle runs Wind::fly (wind.hpp:28-117) against the
//           heights as they were at the start of the step (nothing writes H
//           during this kernel). Its erosion/deposition exchange
//           (wind.hpp:110-112) is added to the delta map D and the cascade it
//           owes its cell (wind.hpp:114) to the visit map C, with integer
//           atomics.
//  cascade  World::cascade (world.hpp:79-153) for every owed visit, in a fixed
//           conflict-free order: four passes over 32x32 tiles by tile colour
//           (tx%2, tz%2); inside a tile, nine cell colours (x%3, z%3) with a
//           block barrier between them. Cells of one colour, and tiles of one
//           colour, touch disjoint 3x3 neighbourhoods, so every cascade sees
//           the latest heights, as in the reference, and the whole step has
//           one order independent of thread scheduling.
// Every exchange and transfer moves the same integer amount out of one place
// and into another, so heights + carried + exported sediment is conserved
// exactly; the result is bitwise reproducible.
//
// Heights are Q(31-f).f fixed point (f = frac_bits); tracks are 64-bit
// integers in units of 2^-32; particle sediment is fixed point like heights.
// Survivors of a step are compacted into the other particle buffer with a
// warp ballot and one atomic per warp.
#include "swe_device.cuh"
#include "swe_kernels.h"

namespace swe {
namespace {

constexpr float kTwo32 = 4294967296.0f;
constexpr float kInvTwo32 = 2.3283064365386963e-10f;
constexpr float kSqrt2 = 1.41421354f;  // sqrtf(2.0f), correctly rounded

__device__ __forceinline__ float fx2f(int32_t q, float inv) { return __int2float_rn(q) * inv; }

__device__ __forceinline__ int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wrap_sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void k_height_to_fixed(const float* __restrict__ H, int32_t* __restrict__ Q, Consts c, Counters* cnt) {
  const long n = (long)c.nx * c.nz;
  unsigned bad = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float v = H[i] * c.scale;
    if (!(fabsf(v) < 1073741824.0f)) bad = 1;
    Q[i] = to_fixed(v);
  }
  if (bad) atomicOr(&cnt->status, 0x2u);  // SWE_STATUS_RANGE
}

__global__ void k_par_spawn(ParallelBuffers B, Consts c, uint32_t seed_lo, uint32_t seed_hi, Counters* cnt,
                            int particles, long n_cells) {
  const unsigned long long cyc = cnt->cycle;
  const uint32_t c_lo = (uint32_t)cyc, c_hi = (uint32_t)(cyc >> 32);
  const long total = n_cells > particles ? n_cells : particles;
  const ParticleSoA S = B.state[0];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    if (i < n_cells) {
      B.tq[0][i] = 0; B.tq[1][i] = 0; B.tq[2][i] = 0; B.tq[3][i] = 0;
    }
    if (i < particles) {
      // Uniform cell plus a 1/1000-quantised offset, as world.hpp:52-54.
      const uint4 u = philox4x32((uint32_t)i, 0xFFFFFFFFu, c_lo, c_hi, seed_lo, seed_hi);
      const int x = (int)(u.x % (uint32_t)c.nx);
      const int z = (int)(u.y % (uint32_t)c.nz);
      const int fxq = (int)(u.z % 1000u);
      const int fzq = (int)(u.w % 1000u);
      S.id[i] = (int)i;
      S.age[i] = 0;
      S.px[i] = (float)x + (float)fxq / 1000.0f;
      S.py[i] = 0.0f;
      S.pz[i] = (float)z + (float)fzq / 1000.0f;
      S.vx[i] = 0.0f; S.vy[i] = 0.0f; S.vz[i] = 0.0f;
      S.sed_q[i] = 0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt->live[0] = particles;
    cnt->live[1] = 0;
    cnt->particles += (unsigned long long)particles;
  }
}

// One Wind::fly step of every live particle against the step-start heights
// H. The exchange with the cell goes to the delta map D and the visit to the
// count map C; the cascade runs afterwards in k_par_cascade.
__global__ void __launch_bounds__(256) k_par_fly(ParallelBuffers B, Consts c, uint32_t seed_lo, uint32_t seed_hi,
                                                 Counters* cnt, int step) {
  const int in = step & 1, outp = in ^ 1;
  const int count = cnt->live[in];
  if (count == 0) return;
  const unsigned long long cyc = cnt->cycle;
  const uint32_t c_lo = (uint32_t)cyc, c_hi = (uint32_t)(cyc >> 32);
  const ParticleSoA S = B.state[in];
  const ParticleSoA Dst = B.state[outp];
  const int32_t* __restrict__ H = B.hq;
  const int nx = c.nx, nz = c.nz;
  const float inv = c.inv_scale;

  long long exported = 0;
  unsigned long long steps = 0;
  unsigned status = 0;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;

  for (int base = warp * 32; base < count; base += nwarps * 32) {
    const int i = base + lane;
    bool alive = false;
    int id = 0, age = 0, sed_q = 0;
    float px = 0, py = 0, pz = 0, vx = 0, vy = 0, vz = 0;
    if (i < count) {
      id = S.id[i]; age = S.age[i]; sed_q = S.sed_q[i];
      px = S.px[i]; py = S.py[i]; pz = S.pz[i];
      vx = S.vx[i]; vy = S.vy[i]; vz = S.vz[i];
      const float sed = fx2f(sed_q, inv);
      const bool inrange = fabsf(px) < 1073741824.0f && fabsf(pz) < 1073741824.0f;
      const int ix = inrange ? (int)roundf(px) : -1;
      const int iz = inrange ? (int)roundf(pz) : -1;
      bool dies = ix < 0 || iz < 0 || ix >= nx || iz >= nz;
      if (!dies) {
        const bool vx0 = ix > 0, vx2 = ix + 1 < nx, vz0 = iz > 0, vz2 = iz + 1 < nz;
        const long ci = (long)ix * nz + iz;
        const float h11 = fx2f(__ldg(H + ci), inv);
        const float h01 = vx0 ? fx2f(__ldg(H + ci - nz), inv) : 0.0f;
        const float h21 = vx2 ? fx2f(__ldg(H + ci + nz), inv) : 0.0f;
        const float h10 = vz0 ? fx2f(__ldg(H + ci - 1), inv) : 0.0f;
        const float h12 = vz2 ? fx2f(__ldg(H + ci + 1), inv) : 0.0f;

        // quad::_normal (cellpool.h:200-223) on the step-start heights.
        V3 n = v3(0.0f, 0.0f, 0.0f);
        const V3 s = v3(1.0f, c.mapscale, 1.0f);
        if (vx2 && vz2) n = add(n, cross(mulv(s, v3(0.0f, h12 - h11, 1.0f)), mulv(s, v3(1.0f, h21 - h11, 0.0f))));
        if (vx0 && vz0) n = add(n, cross(mulv(s, v3(0.0f, h10 - h11, -1.0f)), mulv(s, v3(-1.0f, h01 - h11, 0.0f))));
        if (vx2 && vz0) n = add(n, cross(mulv(s, v3(1.0f, h21 - h11, 0.0f)), mulv(s, v3(0.0f, h10 - h11, -1.0f))));
        if (vx0 && vz2) n = add(n, cross(mulv(s, v3(-1.0f, h01 - h11, 0.0f)), mulv(s, v3(0.0f, h12 - h11, 1.0f))));
        if (length(n) > 0.0f) n = normalize(n);

        if (age == 0 || py < h11) py = h11;
        if (age++ > c.max_age) dies = true;
        if (!dies) {
          float hfac = expf_poly(-(py - h11) / c.boundarylayer);
          if (hfac < 0.0f) hfac = 0.0f;
          const V3 ps = v3(c.px, c.py, c.pz);
          V3 sp = v3(vx, vy, vz);
          float shadow = dot(normalize(ps), n);
          if (shadow < 0.0f) shadow = 0.0f;
          shadow = 1.0f - shadow;
          sp = add(sp, smul(0.05f, sub(smul(0.1f + 0.9f * shadow, ps), sp)));
          if (py > h11) sp.y -= c.gravity * sed;
          float collision = -dot(normalize(sp), n);
          if (collision < 0.0f) collision = 0.0f;
          const V3 rs = cross(n, cross(smul(1.0f - collision, sp), n));
          sp = add(sp, smul(0.9f, sub(smul(shadow, mix(ps, rs, shadow * hfac)), sp)));
          const uint4 u = philox4x32((uint32_t)id, (uint32_t)step, c_lo, c_hi, seed_lo, seed_hi);
          const float rx = (float)(int)(u.x % 1001u), ry = (float)(int)(u.y % 1001u), rz = (float)(int)(u.z % 1001u);
          sp = add(sp, divs(smul(0.1f * hfac * collision, subs(v3(rx, ry, rz), 500.0f)), 500.0f));
          const float drag = 1.0f - 0.3f * sed;
          sp = v3(sp.x * drag, sp.y * drag, sp.z * drag);
          const float npx = px + sp.x, npy = py + sp.y, npz = pz + sp.z;

          float force = -dot(normalize(sp), n) * length(sp);
          if (force < 0.0f) force = 0.0f;
          const float lift = (1.0f - collision) * length(sp);
          const float capacity = force * hfac + 0.02f * lift * hfac;
          const float diff = capacity - sed;
          if (!(isfinite(diff) && isfinite(npx) && isfinite(npy) && isfinite(npz))) {
            status |= 0x1u;  // SWE_STATUS_NONFINITE: retire the particle, no writes
            dies = true;
          } else {
            // Tracks of the pre-move cell (wind.hpp:93-96).
            atomicAdd((unsigned long long*)&B.tq[0][ci], (unsigned long long)to_fixed64(sed * kTwo32));
            atomicAdd((unsigned long long*)&B.tq[1][ci], (unsigned long long)to_fixed64(sp.x * kTwo32));
            atomicAdd((unsigned long long*)&B.tq[2][ci], (unsigned long long)to_fixed64(sp.y * kTwo32));
            atomicAdd((unsigned long long*)&B.tq[3][ci], (unsigned long long)to_fixed64(sp.z * kTwo32));
            // Exchange with the cell (wind.hpp:110-112), in fixed point, and
            // one cascade owed to the cell (wind.hpp:114).
            const int32_t ex_q = to_fixed(c.suspension * diff * c.scale);
            atomicAdd(B.dq + ci, -ex_q);
            atomicAdd(B.visits + ci, 1);
            sed_q = wrap_add(sed_q, ex_q);
            px = npx; py = npy; pz = npz;
            vx = sp.x; vy = sp.y; vz = sp.z;
            alive = true;
            steps++;
          }
        }
      }
      if (!alive) exported += sed_q;
    }
    // Compact survivors into the other buffer: one atomic per warp.
    const unsigned mask = __ballot_sync(0xffffffffu, alive);
    int slot0 = 0;
    if (lane == 0 && mask) slot0 = atomicAdd(&cnt->live[outp], __popc(mask));
    slot0 = __shfl_sync(0xffffffffu, slot0, 0);
    if (alive) {
      const int o = slot0 + __popc(mask & ((1u << lane) - 1u));
      Dst.id[o] = id; Dst.age[o] = age; Dst.sed_q[o] = sed_q;
      Dst.px[o] = px; Dst.py[o] = py; Dst.pz[o] = pz;
      Dst.vx[o] = vx; Dst.vy[o] = vy; Dst.vz[o] = vz;
    }
  }
  exported = warp_sum(exported);
  steps = warp_sum(steps);
  status = __reduce_or_sync(0xffffffffu, status);
  if (lane == 0) {
    if (exported) atomicAdd((unsigned long long*)&cnt->exported_q, (unsigned long long)exported);
    if (steps) atomicAdd(&cnt->particle_steps, steps);
    if (status) atomicOr(&cnt->status, status);
  }
}

constexpr int kTile = 32;          // cells per tile side
constexpr int kLs = kTile + 2;     // with the one-cell halo
constexpr int kCascadeThreads = 128;

// World::cascade (world.hpp:79-153) in fixed point on the shared-memory
// tile: neighbours in the reference's order, stable descending by their
// current height (original order breaks ties), each moving half the excess
// over the slope limit. Ranks instead of a sort keep everything in
// registers.
__device__ __forceinline__ int cascade_smem(int32_t (*L)[kLs], int li, int lj, bool vx0, bool vx2, bool vz0,
                                            bool vz2, const Consts& c) {
  const bool val[8] = {vx0 && vz0, vx0, vx0 && vz2, vz0, vz2, vx2 && vz0, vx2, vx2 && vz2};
  int32_t key[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int a = k < 3 ? 0 : (k < 5 ? 1 : 2);
    const int b = (k == 0 || k == 3 || k == 5) ? 0 : ((k == 1 || k == 6) ? 1 : 2);
    key[k] = L[li + a - 1][lj + b - 1];
  }
  int rank[8];
  int num = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    num += val[k] ? 1 : 0;
    int r = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      if (j == k) continue;
      r += (val[j] && (key[j] > key[k] || (j < k && key[j] == key[k]))) ? 1 : 0;
    }
    rank[k] = val[k] ? r : 8;
  }
  int32_t hc = L[li][lj];
  int32_t dl[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int transfers = 0;
  for (int r = 0; r < num; r++) {
    int32_t kq = 0;
    float d = 1.0f;
    int sel = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      if (rank[k] == r) {
        kq = key[k];
        d = (k == 1 || k == 3 || k == 4 || k == 6) ? 1.0f : kSqrt2;
        sel = k;
      }
    }
    const long long dq = (long long)hc - (long long)kq;
    if (dq == 0) continue;
    const float excess = fabsf(__ll2float_rn(dq) * c.inv_scale) - d * c.maxdiff;
    if (excess <= 0.0f) continue;
    const int32_t tq = to_fixed(c.settling * excess / 2.0f * c.scale);
    const int32_t sgn = dq > 0 ? tq : -tq;
    hc = wrap_sub(hc, sgn);
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (k == sel) dl[k] = wrap_add(dl[k], sgn);
    transfers++;
  }
  L[li][lj] = hc;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if (dl[k] != 0) {
      const int a = k < 3 ? 0 : (k < 5 ? 1 : 2);
      const int b = (k == 0 || k == 3 || k == 5) ? 0 : ((k == 1 || k == 6) ? 1 : 2);
      L[li + a - 1][lj + b - 1] = wrap_add(L[li + a - 1][lj + b - 1], dl[k]);
    }
  }
  return transfers;
}

// One cascade pass over the tiles of colour (color>>1, color&1). A block
// loads its 32x32 tile plus halo (heights + pending exchange deltas), runs
// every owed cascade colour by colour (x%3, z%3) with a block barrier
// between colours, and writes the tile back: own cells absorb their deltas,
// halo cells go back without theirs (their own tile absorbs them).
__global__ void __launch_bounds__(kCascadeThreads) k_par_cascade(ParallelBuffers B, Consts c, Counters* cnt,
                                                                 int step, int color, int tiles_z) {
  const int surv = cnt->live[(step + 1) & 1];
  if (color == 0 && blockIdx.x == 0 && threadIdx.x == 0) cnt->live[step & 1] = 0;
  if (surv == 0) return;
  __shared__ int32_t L[kLs][kLs];
  const int nx = c.nx, nz = c.nz;
  const int tx = (color >> 1) + 2 * (blockIdx.x / tiles_z);
  const int tz = (color & 1) + 2 * (blockIdx.x % tiles_z);
  const int x0 = tx * kTile, z0 = tz * kTile;
  int32_t* __restrict__ H = B.hq;
  int32_t* __restrict__ Dq = B.dq;
  int32_t* __restrict__ V = B.visits;

  for (int idx = threadIdx.x; idx < kLs * kLs; idx += kCascadeThreads) {
    const int i = idx / kLs, j = idx % kLs;
    const int x = x0 + i - 1, z = z0 + j - 1;
    int32_t v = 0;
    if (x >= 0 && z >= 0 && x < nx && z < nz) {
      const long g = (long)x * nz + z;
      v = wrap_add(H[g], Dq[g]);
    }
    L[i][j] = v;
  }
  __syncthreads();

  int transfers = 0;
  const int t = threadIdx.x;
  const int m = t / 11, l = t % 11;
#pragma unroll 1
  for (int col = 0; col < 9; col++) {
    const int a = col / 3, b = col % 3;
    const int i = ((a - x0 % 3) + 3) % 3 + 3 * m;
    const int j = ((b - z0 % 3) + 3) % 3 + 3 * l;
    const int x = x0 + i, z = z0 + j;
    if (t < 121 && i < kTile && j < kTile && x < nx && z < nz) {
      const int visits = V[(long)x * nz + z];
      for (int r = 0; r < visits; r++)
        transfers += cascade_smem(L, i + 1, j + 1, x > 0, x + 1 < nx, z > 0, z + 1 < nz, c);
    }
    __syncthreads();
  }

  for (int idx = threadIdx.x; idx < kLs * kLs; idx += kCascadeThreads) {
    const int i = idx / kLs, j = idx % kLs;
    const int x = x0 + i - 1, z = z0 + j - 1;
    if (x < 0 || z < 0 || x >= nx || z >= nz) continue;
    const long g = (long)x * nz + z;
    const bool own = i >= 1 && j >= 1 && i <= kTile && j <= kTile;
    if (own) {
      H[g] = L[i][j];
      Dq[g] = 0;
      V[g] = 0;
    } else {
      H[g] = wrap_sub(L[i][j], Dq[g]);
    }
  }
  const int tw = warp_sum(transfers);
  if ((threadIdx.x & 31) == 0 && tw) atomicAdd(&cnt->transfers, (unsigned long long)tw);
}

// Tracks to float, EMA (world.hpp:70-76), heights to float; count the cycle.
__global__ void k_par_ema(ParallelBuffers B, Fields F, Consts c, Counters* cnt, long n) {
  unsigned bad = 0;
  const float lrate = c.lrate;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float t = __ll2float_rn(B.tq[k][i]) * kInvTwo32;
      F.f[5 + k][i] = t;
      F.f[1 + k][i] = (1.0f - lrate) * F.f[1 + k][i] + lrate * t;
    }
    const int32_t q = B.hq[i];
    if (q > 1073741823 || q < -1073741823) bad = 1;
    F.f[0][i] = fx2f(q, c.inv_scale);
  }
  if (bad) atomicOr(&cnt->status, 0x2u);
  if (blockIdx.x == 0 && threadIdx.x == 0) cnt->cycle += 1;
}

__global__ void k_sum_fixed(const int32_t* __restrict__ hq, long n, long long* out) {
  long long acc = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) acc += hq[i];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) atomicAdd((unsigned long long*)out, (unsigned long long)acc);
}

inline int sweep_grid(long n) {
  long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

void launch_height_to_fixed(const float* height, int32_t* q, const Consts& c, Counters* cnt, cudaStream_t s) {
  k_height_to_fixed<<<sweep_grid((long)c.nx * c.nz), 256, 0, s>>>(height, q, c, cnt);
}

void launch_par_spawn(const ParallelBuffers& B, const Consts& c, uint64_t seed, Counters* cnt, int particles,
                      long n_cells, cudaStream_t s) {
  const long total = n_cells > particles ? n_cells : particles;
  k_par_spawn<<<sweep_grid(total), 256, 0, s>>>(B, c, (uint32_t)seed, (uint32_t)(seed >> 32), cnt, particles,
                                                n_cells);
}

void launch_par_fly(const ParallelBuffers& B, const Consts& c, uint64_t seed, Counters* cnt, int step, int grid,
                    cudaStream_t s) {
  k_par_fly<<<grid, 256, 0, s>>>(B, c, (uint32_t)seed, (uint32_t)(seed >> 32), cnt, step);
}

void launch_par_cascade(const ParallelBuffers& B, const Consts& c, Counters* cnt, int step, cudaStream_t s) {
  const int tiles_x = (c.nx + kTile - 1) / kTile, tiles_z = (c.nz + kTile - 1) / kTile;
  for (int color = 0; color < 4; color++) {
    const int cx = color >> 1, cz = color & 1;
    const int gx = (tiles_x - cx + 1) / 2, gz = (tiles_z - cz + 1) / 2;
    if (gx <= 0 || gz <= 0) {
      // No tile of this colour; pass 0 still resets the live counter.
      if (color == 0) k_par_cascade<<<1, kCascadeThreads, 0, s>>>(B, c, cnt, step, color, 1);
      continue;
    }
    k_par_cascade<<<gx * gz, kCascadeThreads, 0, s>>>(B, c, cnt, step, color, gz);
  }
}

void launch_par_ema(const ParallelBuffers& B, const Fields& F, const Consts& c, Counters* cnt, long n_cells,
                    cudaStream_t s) {
  k_par_ema<<<sweep_grid(n_cells), 256, 0, s>>>(B, F, c, cnt, n_cells);
}

void launch_sum_fixed(const int32_t* hq, long n, long long* out, cudaStream_t s) {
  k_sum_fixed<<<sweep_grid(n), 256, 0, s>>>(hq, n, out);
}

int par_step_grid(int device) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_par_fly, 256, 0);
  if (per_sm < 1) per_sm = 1;
  if (sms < 1) sms = 1;
  return sms * per_sm;
}

}  // namespace swe
