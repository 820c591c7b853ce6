// Parallel fixed-point erosion: all particles of an erode cycle fly together.
//
// One erode cycle (the World::erode(P) call, world.hpp:36-77) is ONE
// persistent cooperative kernel, k_par_cycle, whose phases are separated by a
// grid barrier:
//   spawn     zero the track accumulators, spawn the first `lanes` of the
//             cycle's P particles
//   per step (until every particle of the cycle has flown):
//     fly     every live particle runs Wind::fly (wind.hpp:28-117) against
//             the heights as they were at the start of the step (nothing
//             writes H in this phase). Its erosion/deposition exchange
//             (wind.hpp:110-112) is added to the delta map D and the cascade
//             it owes its cell (wind.hpp:114) to the visit map C, with integer
//             atomics; survivors are compacted into the other particle buffer,
//             and the lanes of the particles that died take the cycle's next
//             particles (warp-cooperative spawning), which fly from the next
//             step. Few lanes keep each flight on a nearly static map, as in
//             the sequential reference; all P at once is fastest.
//     colour  nine phases, cell colour (x%3, z%3). Colour 0 first adds the
//             pending exchange deltas (H += D, D = 0) of the 3x3 block around
//             each colour-0 cell; these blocks tile the map, so that is the
//             same as adding every delta before the first cascade. Then, in
//             every colour phase, every cell with C > 0 runs
//             World::cascade (world.hpp:79-153) up to C times on the current
//             heights, stopping once a cascade moves nothing (repeating it
//             could not change anything). Cells of one colour touch disjoint
//             3x3 neighbourhoods, so no two threads touch the same cell.
//   ema       tracks -> float, EMA of massflow/momentum (world.hpp:70-76),
//             fixed-point heights -> float.
// Every exchange and transfer moves the same integer amount out of one place
// and into another, so heights + carried + exported sediment is conserved
// exactly, and the phase order makes the result bitwise reproducible.
//
// Heights are Q(31-f).f fixed point (f = frac_bits); tracks are 64-bit
// integers in units of 2^-32; particle sediment is fixed point like heights.
//
// The grid barrier spins with an explicit deadline: a block that waits longer
// than the wait limit (Consts::wait_ns, 2 s by default) sets
// SWE_STATUS_TIMEOUT and an abort flag, and every block then leaves the
// kernel at its next barrier, so the kernel always ends.
#include <algorithm>
#include <vector>

#include "swe_device.cuh"
#include "swe_kernels.h"

namespace swe {
namespace {

constexpr float kTwo32 = 4294967296.0f;
constexpr float kInvTwo32 = 2.3283064365386963e-10f;
constexpr float kSqrt2 = 1.41421354f;  // sqrtf(2.0f), correctly rounded
constexpr int kCycleThreads = 256;
constexpr int kCycleBlocksPerSm = 4;  // 64 registers per thread, no spills
constexpr unsigned long long kBarrierLimitNs = 2000000000ull;  // the default wait deadline

__host__ __device__ __forceinline__ unsigned long long wait_limit(const Consts& c) {
  return c.wait_ns ? c.wait_ns : kBarrierLimitNs;
}

__device__ __forceinline__ float fx2f(int32_t q, float inv) { return __int2float_rn(q) * inv; }
__device__ __forceinline__ int32_t wrap_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
__device__ __forceinline__ int32_t wrap_sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Grid-wide barrier of a cooperative launch (all blocks co-resident), one
// arrival atomic per block: every block adds 1 to the flip counter but block
// 0, which adds 2^31 - (blocks - 1), so the counter's top bit flips exactly
// when the last block arrives; each block waits for the flip relative to the
// value its own arrival returned (release/acquire atomics, no separate
// fences, no generation word to read first or to publish last). Thread 0
// arrives for its block; the block barriers before and after carry the rest
// of the block's threads. Every wait has a deadline (`limit`), after which the
// block sets SWE_STATUS_TIMEOUT and the abort flag; returns false if the
// kernel must stop.
__device__ bool grid_sync(GridBarrier* gb, unsigned int* status, unsigned long long limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1) : 1u;
    const unsigned old = atom_add_acq_rel(&gb->flip, add);
    const unsigned long long t0 = global_ns();
    while (((ld_acquire(&gb->flip) ^ old) & 0x80000000u) == 0) {
      if (ld_acquire(&gb->abort)) {
        ok = 0;
        break;
      }
      if (global_ns() - t0 > limit) {
        atomicOr(status, 0x8u);  // SWE_STATUS_TIMEOUT
        atomicExch(&gb->abort, 1u);
        ok = 0;
        break;
      }
    }
    if (ld_acquire(&gb->abort)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// A grid barrier of one 64-bit atomic per block whose arrivals also add up
// one count per block. The word sums[phase] (phase = step mod 3, one 128-byte
// line each) holds the arrivals in its high half and the counts in its low
// half; a block adds 2^32 + its count and waits until the high half shows
// every block. *below gets the counts of the blocks whose arrivals landed
// before this one's (an arrival order standing in for a block order),
// *total the sum over all blocks, from the same word. Block 0 clears the
// word of phase + 1 mod 3 before it arrives: that word's last total was read
// two barriers ago, and its next arrivals come after this barrier. The poll
// reads the abort flag (relaxed) ahead of the word (acquire), so that the two
// loads overlap; the last block to arrive reads neither.
__device__ __forceinline__ unsigned long long atom_add_acq_rel64(unsigned long long* p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}

__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned ld_relaxed32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ bool grid_sync_sum(GridBarrier* gb, unsigned int* status, unsigned long long limit, unsigned phase,
                              unsigned mine, unsigned* below, unsigned* total) {
  __shared__ int s_ok;
  __shared__ unsigned s_below, s_total;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned long long* word = reinterpret_cast<unsigned long long*>(&gb->sums[32 * phase]);
    if (blockIdx.x == 0) {
      unsigned long long* next = reinterpret_cast<unsigned long long*>(&gb->sums[32 * (phase == 2 ? 0 : phase + 1)]);
      asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(next), "l"(0ull) : "memory");
    }
    const unsigned long long add = (1ull << 32) | mine;
    const unsigned long long old = atom_add_acq_rel64(word, add);
    const unsigned long long all = (unsigned long long)gridDim.x << 32;
    unsigned long long v = old + add;
    unsigned long long t0 = 0;
    for (unsigned i = 0; (v & 0xFFFFFFFF00000000ull) != all; i++) {
      const unsigned ab = ld_relaxed32(&gb->abort);
      v = ld_acquire64(word);
      if (ab) {
        ok = 0;
        break;
      }
      if ((i & 15u) == 15u) {
        const unsigned long long now = global_ns();
        if (t0 == 0) {
          t0 = now;
        } else if (now - t0 > limit) {
          atomicOr(status, 0x8u);  // SWE_STATUS_TIMEOUT
          atomicExch(&gb->abort, 1u);
          ok = 0;
          break;
        }
      }
    }
    s_below = (unsigned)old;
    s_total = (unsigned)v;
    s_ok = ok;
  }
  __syncthreads();
  *below = s_below;
  *total = s_total;
  return s_ok != 0;
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

struct CycleArgs {
  ParallelBuffers B;
  Fields F;
  Consts c;
  uint32_t seed_lo, seed_hi;
  Counters* cnt;
  GridBarrier* gb;
  int particles;  // particles of the cycle
  int lanes;      // particles in flight at once
  int spread;     // bounded lanes: a CTA's lanes spread over its warps (lane l of warp w first) instead of packed
};

// Per-thread tallies of the colour phases.
template <class U>
struct CascadeTally {
  U transfers = 0;             // transfers that moved a non-zero amount
  U cascades = 0;              // World::cascade evaluations
  U cells = 0;                 // cells with owed cascades
  unsigned int max_iters = 0;  // most cascades one cell ran in one step
};
using CascadeStats = CascadeTally<unsigned long long>;

// One particle at its spawn point: a uniform cell plus a 1/1000-quantised
// offset (world.hpp:52-54), drawn from Philox counter (id, 0xFFFFFFFF, cycle).
__device__ __forceinline__ void spawn_one(const CycleArgs& A, const ParticleSoA& S, int slot, int id, uint32_t c_lo,
                                          uint32_t c_hi) {
  const uint4 u = philox4x32((uint32_t)id, 0xFFFFFFFFu, c_lo, c_hi, A.seed_lo, A.seed_hi);
  const int x = (int)(u.x % (uint32_t)A.c.nx);
  const int z = (int)(u.y % (uint32_t)A.c.nz);
  const int fxq = (int)(u.z % 1000u);
  const int fzq = (int)(u.w % 1000u);
  S.id[slot] = id;
  S.age[slot] = 0;
  S.px[slot] = (float)x + (float)fxq / 1000.0f;
  S.py[slot] = 0.0f;
  S.pz[slot] = (float)z + (float)fzq / 1000.0f;
  S.vx[slot] = 0.0f; S.vy[slot] = 0.0f; S.vz[slot] = 0.0f;
  S.sed_q[slot] = 0;
}

// Spawn phase: zero the tracks and spawn the first min(lanes, particles)
// particles of the cycle.
__device__ void spawn_phase(const CycleArgs& A, uint32_t c_lo, uint32_t c_hi) {
  const long n = (long)A.c.nx * A.c.nz;
  const int first = A.lanes < A.particles ? A.lanes : A.particles;
  const long total = n > first ? n : first;
  const ParticleSoA S = A.B.state[0];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    if (i < n) {
      A.B.tq[0][i] = 0; A.B.tq[1][i] = 0; A.B.tq[2][i] = 0; A.B.tq[3][i] = 0;
    }
    if (i < first) spawn_one(A, S, (int)i, (int)i, c_lo, c_hi);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    A.cnt->live[0] = first;
    A.cnt->live[1] = 0;
    A.cnt->refill[0] = 0;
    A.cnt->refill[1] = 0;
    A.cnt->next_id[0] = first;
    A.cnt->next_id[1] = first;
    A.cnt->particles += (unsigned long long)A.particles;
  }
}

// Freed lanes take the cycle's next particles: ids id0 .. id0+k-1 go to
// slots slot0 .. slot0+k-1 of state buffer `buf`; they fly from the next step.
__device__ void refill_lanes(const CycleArgs& A, int buf, int slot0, int id0, int k, uint32_t c_lo, uint32_t c_hi) {
  const ParticleSoA S = A.B.state[buf];
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < k; j += gridDim.x * blockDim.x)
    spawn_one(A, S, slot0 + j, id0 + j, c_lo, c_hi);
}

// One particle in flight.
struct Particle {
  int id, age, sed_q;
  float px, py, pz, vx, vy, vz;
};

// The turbulence draws of a particle's next step (wind.hpp:102-104): keyed
// by (particle, age after the step's increment, cycle), each an integer in
// [0, 1000] as a float. They depend on no height, so a caller may take them
// before the step's heights arrive.
struct Turbulence {
  float rx, ry, rz;
};
__device__ __forceinline__ Turbulence turbulence(const Particle& p, uint32_t c_lo, uint32_t c_hi, uint32_t seed_lo,
                                                 uint32_t seed_hi) {
  const uint4 u = philox4x32((uint32_t)p.id, (uint32_t)(p.age + 1), c_lo, c_hi, seed_lo, seed_hi);
  return Turbulence{(float)(int)(u.x % 1001u), (float)(int)(u.y % 1001u), (float)(int)(u.z % 1001u)};
}

// The cell a particle is over (its position rounded, as ivec2(round(...)),
// wind.hpp:30), or -1 off the map.
__device__ __forceinline__ long particle_cell(const Consts& c, const Particle& p, int& ix, int& iz) {
  const bool inrange = fabsf(p.px) < 1073741824.0f && fabsf(p.pz) < 1073741824.0f;
  ix = inrange ? (int)roundf(p.px) : -1;
  iz = inrange ? (int)roundf(p.pz) : -1;
  if (ix < 0 || iz < 0 || ix >= c.nx || iz >= c.nz) return -1;
  return (long)ix * c.nz + iz;
}

// One Wind::fly step (wind.hpp:28-117) of particle p over cell ci = (ix, iz),
// given the step-start heights of the cell and of its x-1, x+1, z-1, z+1
// neighbours (fixed point; those off the map are not used). A survivor adds
// its tracks (wind.hpp:93-96) and its exchange with the cell
// (wind.hpp:110-112) to the accumulators (exchange into dq), moves, and ci is
// returned; the caller records the cascade it owes the cell (wind.hpp:114). A
// particle that dies returns -1 and writes nothing (its sediment is exported).
__device__ __forceinline__ long fly_from(const Consts& c, const ParallelBuffers& B, int32_t* dq, long ci, int ix,
                                         int iz, int32_t q11, int32_t q01, int32_t q21, int32_t q10, int32_t q12,
                                         const Turbulence& tb, Particle& p, unsigned& status) {
  const int nx = c.nx, nz = c.nz;
  const float inv = c.inv_scale;
  const float sed = fx2f(p.sed_q, inv);
  const bool vx0 = ix > 0, vx2 = ix + 1 < nx, vz0 = iz > 0, vz2 = iz + 1 < nz;
  const float h11 = fx2f(q11, inv);
  const float h01 = vx0 ? fx2f(q01, inv) : 0.0f;
  const float h21 = vx2 ? fx2f(q21, inv) : 0.0f;
  const float h10 = vz0 ? fx2f(q10, inv) : 0.0f;
  const float h12 = vz2 ? fx2f(q12, inv) : 0.0f;

  // quad::_normal (cellpool.h:200-223) on the step-start heights.
  V3 n = v3(0.0f, 0.0f, 0.0f);
  const V3 s = v3(1.0f, c.mapscale, 1.0f);
  if (vx2 && vz2) n = add(n, cross(mulv(s, v3(0.0f, h12 - h11, 1.0f)), mulv(s, v3(1.0f, h21 - h11, 0.0f))));
  if (vx0 && vz0) n = add(n, cross(mulv(s, v3(0.0f, h10 - h11, -1.0f)), mulv(s, v3(-1.0f, h01 - h11, 0.0f))));
  if (vx2 && vz0) n = add(n, cross(mulv(s, v3(1.0f, h21 - h11, 0.0f)), mulv(s, v3(0.0f, h10 - h11, -1.0f))));
  if (vx0 && vz2) n = add(n, cross(mulv(s, v3(-1.0f, h01 - h11, 0.0f)), mulv(s, v3(0.0f, h12 - h11, 1.0f))));
  if (length(n) > 0.0f) n = normalize(n);

  float py = p.py;
  if (p.age == 0 || py < h11) py = h11;
  if (p.age++ > c.max_age) return -1;
  float hfac = expf_poly(-(py - h11) / c.boundarylayer);
  if (hfac < 0.0f) hfac = 0.0f;
  const V3 ps = v3(c.px, c.py, c.pz);
  V3 sp = v3(p.vx, p.vy, p.vz);
  float shadow = dot(normalize(ps), n);
  if (shadow < 0.0f) shadow = 0.0f;
  shadow = 1.0f - shadow;
  sp = add(sp, smul(0.05f, sub(smul(0.1f + 0.9f * shadow, ps), sp)));
  if (py > h11) sp.y -= c.gravity * sed;
  float collision = -dot(normalize(sp), n);
  if (collision < 0.0f) collision = 0.0f;
  const V3 rs = cross(n, cross(smul(1.0f - collision, sp), n));
  sp = add(sp, smul(0.9f, sub(smul(shadow, mix(ps, rs, shadow * hfac)), sp)));
  // turbulence draws keyed by (particle, age after this step's increment)
  sp = add(sp, divs(smul(0.1f * hfac * collision, subs(v3(tb.rx, tb.ry, tb.rz), 500.0f)), 500.0f));
  const float drag = 1.0f - 0.3f * sed;
  sp = v3(sp.x * drag, sp.y * drag, sp.z * drag);
  const float npx = p.px + sp.x, npy = py + sp.y, npz = p.pz + sp.z;

  float force = -dot(normalize(sp), n) * length(sp);
  if (force < 0.0f) force = 0.0f;
  const float lift = (1.0f - collision) * length(sp);
  const float capacity = force * hfac + 0.02f * lift * hfac;
  const float diff = capacity - sed;
  if (!(isfinite(diff) && isfinite(npx) && isfinite(npy) && isfinite(npz))) {
    status |= 0x1u;  // SWE_STATUS_NONFINITE: retire the particle, no writes
    return -1;
  }
  // Tracks of the pre-move cell (wind.hpp:93-96).
  atomicAdd((unsigned long long*)&B.tq[0][ci], (unsigned long long)to_fixed64(sed * kTwo32));
  atomicAdd((unsigned long long*)&B.tq[1][ci], (unsigned long long)to_fixed64(sp.x * kTwo32));
  atomicAdd((unsigned long long*)&B.tq[2][ci], (unsigned long long)to_fixed64(sp.y * kTwo32));
  atomicAdd((unsigned long long*)&B.tq[3][ci], (unsigned long long)to_fixed64(sp.z * kTwo32));
  // Exchange with the cell (wind.hpp:110-112), in fixed point.
  const int32_t ex_q = to_fixed(c.suspension * diff * c.scale);
  atomicAdd(dq + ci, -ex_q);
  p.sed_q = wrap_add(p.sed_q, ex_q);
  p.px = npx; p.py = npy; p.pz = npz;
  p.vx = sp.x; p.vy = sp.y; p.vz = sp.z;
  return ci;
}

// The whole step, reading the heights from the int32 map H.
__device__ __forceinline__ long fly_particle(const Consts& c, const ParallelBuffers& B, const int32_t* H,
                                             uint32_t c_lo, uint32_t c_hi, uint32_t seed_lo, uint32_t seed_hi,
                                             Particle& p, unsigned& status) {
  int ix, iz;
  const long ci = particle_cell(c, p, ix, iz);
  if (ci < 0) return -1;
  const int nz = c.nz;
  // five unconditional loads (a missing neighbour reads the cell itself)
  const int32_t q11 = H[ci];
  const int32_t q01 = H[ix > 0 ? ci - nz : ci];
  const int32_t q21 = H[ix + 1 < c.nx ? ci + nz : ci];
  const int32_t q10 = H[iz > 0 ? ci - 1 : ci];
  const int32_t q12 = H[iz + 1 < nz ? ci + 1 : ci];
  const Turbulence tb = turbulence(p, c_lo, c_hi, seed_lo, seed_hi);
  return fly_from(c, B, B.dq, ci, ix, iz, q11, q01, q21, q10, q12, tb, p, status);
}

// Fly phase of one step: Wind::fly for every particle in flight against the
// step-start heights; survivors are appended to the other state buffer.
__device__ void fly_phase(const CycleArgs& A, int in, int count, uint32_t c_lo, uint32_t c_hi) {
  const int outp = in ^ 1;
  const ParticleSoA S = A.B.state[in];
  const ParticleSoA Dst = A.B.state[outp];

  long long exported = 0;
  unsigned long long steps = 0;
  unsigned status = 0;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;

  for (int base = warp * 32; base < count; base += nwarps * 32) {
    const int i = base + lane;
    bool alive = false;
    Particle p{};
    if (i < count) {
      p.id = S.id[i]; p.age = S.age[i]; p.sed_q = S.sed_q[i];
      p.px = S.px[i]; p.py = S.py[i]; p.pz = S.pz[i];
      p.vx = S.vx[i]; p.vy = S.vy[i]; p.vz = S.vz[i];
      const long ci = fly_particle(A.c, A.B, A.B.hq, c_lo, c_hi, A.seed_lo, A.seed_hi, p, status);
      if (ci >= 0) {
        atomicAdd(A.B.visits + ci, 1);  // one cascade owed to the cell (wind.hpp:114)
        alive = true;
        steps++;
      } else {
        exported += p.sed_q;
      }
    }
    // Compact survivors into the other buffer: one atomic per warp.
    const unsigned mask = __ballot_sync(0xffffffffu, alive);
    int slot0 = 0;
    if (lane == 0 && mask) slot0 = atomicAdd(&A.cnt->live[outp], __popc(mask));
    slot0 = __shfl_sync(0xffffffffu, slot0, 0);
    if (alive) {
      const int o = slot0 + __popc(mask & ((1u << lane) - 1u));
      Dst.id[o] = p.id; Dst.age[o] = p.age; Dst.sed_q[o] = p.sed_q;
      Dst.px[o] = p.px; Dst.py[o] = p.py; Dst.pz[o] = p.pz;
      Dst.vx[o] = p.vx; Dst.vy[o] = p.vy; Dst.vz[o] = p.vz;
    }
  }
  exported = warp_sum(exported);
  steps = warp_sum(steps);
  status = __reduce_or_sync(0xffffffffu, status);
  if (lane == 0) {
    if (exported) atomicAdd((unsigned long long*)&A.cnt->exported_q, (unsigned long long)exported);
    if (steps) atomicAdd(&A.cnt->particle_steps, steps);
    if (status) atomicOr(&A.cnt->status, status);
  }
}

// Thresholds of one cascade, in both forms used below.
struct CascadeConsts {
  float md1, md2;  // slope limit d*maxdiff of axis / diagonal neighbours
  float hd1, hd2;  // the same in half fixed-point steps (exact power-of-two scaling)
  bool unit;       // settling == 1
};

// Whether a transfer from/to a neighbour at fixed-point height difference dq
// moves a non-zero amount, and how much (World::cascade, world.hpp:132-143:
// transfer = settling * (|diff| - d*maxdiff) / 2). With settling == 1 and
// |dq| < 2^24 the amount rint(((|dq| 2^-f - dmax) * 0.5) * 2^f) equals
// rint(0.5 |dq| - dmax 2^(f-1)) exactly (scaling by powers of two commutes
// with rounding and |dq| is exact in float), and it is non-zero exactly when
// 0.5 |dq| - dmax 2^(f-1) > 0.5.
__device__ __forceinline__ int32_t transfer_q(int32_t dq, bool axis, const CascadeConsts& k, const Consts& c) {
  const int32_t adq = dq < 0 ? -dq : dq;
  if (adq == 0) return 0;
  if (k.unit && adq < (1 << 24)) {
    const float u = fmaf(0.5f, __int2float_rn(adq), axis ? -k.hd1 : -k.hd2);
    return u > 0.5f ? __float2int_rn(u) : 0;
  }
  const float excess = fabsf(__int2float_rn(dq) * c.inv_scale) - (axis ? k.md1 : k.md2);
  if (excess <= 0.0f) return 0;
  return to_fixed(c.settling * excess * 0.5f * c.scale);
}

// World::cascade (world.hpp:79-153) in fixed point on the 3x3 neighbourhood
// N (shared memory, N[3*u+v] is cell (x+u-1, z+v-1)). The in-bounds
// neighbours are ordered by height, largest first, equal heights in the
// reference's neighbour order (std::sort on <= 16 elements is a stable
// insertion sort): the sort keys pack 8*height + (7 - neighbour index) into
// Key (int32 when all nine heights are below 2^27 in magnitude, else int64)
// and go through Knuth's optimal 19-comparator network. The transfers then
// run against the running centre height. A cascade that moves nothing leaves
// the centre unchanged, so a first pass decides that case against the
// current centre in any order and skips the sort. Returns the number of
// transfers that moved a non-zero amount. This general form serves any
// settling and any height range.
template <class Key>
__device__ __forceinline__ int cascade_general(int32_t* N, const bool (&val)[8], const CascadeConsts& kc,
                                               const Consts& c) {
  constexpr int slot[8] = {0, 1, 2, 3, 5, 6, 7, 8};
  constexpr unsigned kAxisMask = 0x5Au;  // neighbours 1, 3, 4, 6 are axis-aligned
  const int32_t h0 = N[4];
  bool any = false;
#pragma unroll
  for (int k = 0; k < 8; k++)
    any |= val[k] && transfer_q(wrap_sub(h0, N[slot[k]]), (kAxisMask >> k) & 1u, kc, c) != 0;
  if (!any) return 0;

  const Key kNone = (Key)1 << (sizeof(Key) * 8 - 1);  // most negative: sorts last
  Key v[8];
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = val[k] ? (Key)N[slot[k]] * 8 + (Key)(7 - k) : kNone;
#define SWE_CE(a, b)                                  \
  {                                                   \
    const Key hi = v[a] > v[b] ? v[a] : v[b];         \
    const Key lo = v[a] > v[b] ? v[b] : v[a];         \
    v[a] = hi;                                        \
    v[b] = lo;                                        \
  }
  SWE_CE(0, 1) SWE_CE(2, 3) SWE_CE(4, 5) SWE_CE(6, 7)
  SWE_CE(0, 2) SWE_CE(1, 3) SWE_CE(4, 6) SWE_CE(5, 7)
  SWE_CE(1, 2) SWE_CE(5, 6) SWE_CE(0, 4) SWE_CE(3, 7)
  SWE_CE(1, 5) SWE_CE(2, 6)
  SWE_CE(1, 4) SWE_CE(3, 6)
  SWE_CE(2, 4) SWE_CE(3, 5)
  SWE_CE(3, 4)
#undef SWE_CE
  int32_t hc = h0;
  int transfers = 0;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    if (v[r] == kNone) break;
    const int k = 7 - (int)(v[r] & 7);
    const int32_t tq = transfer_q(wrap_sub(hc, (int32_t)(v[r] >> 3)), (kAxisMask >> k) & 1u, kc, c);
    if (tq == 0) continue;
    const int32_t sgn = wrap_sub(hc, (int32_t)(v[r] >> 3)) > 0 ? tq : -tq;
    hc = wrap_sub(hc, sgn);
    const int sl = k < 4 ? k : k + 1;
    N[sl] = wrap_add(N[sl], sgn);
    transfers++;
  }
  N[4] = hc;
  return transfers;
}

// The same cascade for the common case, settling == 1 and all nine heights
// within 2^24 fixed-point steps of each other: the centre then stays within
// that range, every |dq| < 2^24, and each transfer is
// rint(0.5 |dq| - dmax 2^(f-1)) when that exceeds 0.5 (see transfer_q).
// Branch-free: the whole chain is selects in registers, and each neighbour's
// new height (its sort key's height plus its transfer) is stored after the
// chain.
__device__ __forceinline__ int cascade_unit(int32_t* N, const bool (&val)[8], float hd1, float hd2) {
  constexpr int slot[8] = {0, 1, 2, 3, 5, 6, 7, 8};
  constexpr unsigned kAxisMask = 0x5Au;
  const int32_t kNone = (int32_t)0x80000000u;
  int32_t h[8];
#pragma unroll
  for (int k = 0; k < 8; k++) h[k] = N[slot[k]];
  const int32_t h0 = N[4];
  bool any = false;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int32_t d = h0 - h[k];
    const int32_t ad = d < 0 ? -d : d;
    const float u = fmaf(0.5f, __int2float_rn(ad), ((kAxisMask >> k) & 1u) ? -hd1 : -hd2);
    any |= val[k] && ad != 0 && u > 0.5f;
  }
  if (!any) return 0;
  int32_t v[8];
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = val[k] ? h[k] * 8 + (7 - k) : kNone;
#define SWE_CE(a, b)                       \
  {                                        \
    const int32_t hi = max(v[a], v[b]);    \
    const int32_t lo = min(v[a], v[b]);    \
    v[a] = hi;                             \
    v[b] = lo;                             \
  }
  SWE_CE(0, 1) SWE_CE(2, 3) SWE_CE(4, 5) SWE_CE(6, 7)
  SWE_CE(0, 2) SWE_CE(1, 3) SWE_CE(4, 6) SWE_CE(5, 7)
  SWE_CE(1, 2) SWE_CE(5, 6) SWE_CE(0, 4) SWE_CE(3, 7)
  SWE_CE(1, 5) SWE_CE(2, 6)
  SWE_CE(1, 4) SWE_CE(3, 6)
  SWE_CE(2, 4) SWE_CE(3, 5)
  SWE_CE(3, 4)
#undef SWE_CE
  int32_t hc = h0;
  int32_t sg[8];
  int transfers = 0;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const bool ok = v[r] != kNone;
    const int k = 7 - (v[r] & 7);
    const int32_t kq = v[r] >> 3;
    const int32_t dq = wrap_sub(hc, kq);  // sentinel entries are masked by `ok`
    const int32_t ad = dq < 0 ? wrap_sub(0, dq) : dq;
    const float u = fmaf(0.5f, __int2float_rn(ad), ((kAxisMask >> k) & 1u) ? -hd1 : -hd2);
    const bool move = ok && ad != 0 && u > 0.5f;
    const int32_t tq = move ? __float2int_rn(u) : 0;
    sg[r] = dq > 0 ? tq : -tq;
    hc = wrap_sub(hc, sg[r]);
    transfers += move ? 1 : 0;
  }
#pragma unroll
  for (int r = 0; r < 8; r++) {
    if (v[r] != kNone) {
      const int k = 7 - (v[r] & 7);
      N[k < 4 ? k : k + 1] = (v[r] >> 3) + sg[r];
    }
  }
  N[4] = hc;
  return transfers;
}

// The cascades a cell owes (world.hpp:79-153, once per visit of the step,
// stopping once a cascade moves nothing) on its 3x3 neighbourhood M, where
// vx0/vx2/vz0/vz2 say whether the x-1, x+1, z-1, z+1 neighbours exist. The
// common case takes the branch-free cascade: settling == 1 and the nine
// heights (of in-bounds cells) within 2^24 steps of each other; cascades keep
// every height inside the initial range.
template <class Tally>
__device__ __forceinline__ void cascade_cell(int32_t* M, bool vx0, bool vx2, bool vz0, bool vz2, int vis,
                                             const CascadeConsts& kc, const Consts& c, Tally& st) {
  const bool val[8] = {vx0 && vz0, vx0, vx0 && vz2, vz0, vz2, vx2 && vz0, vx2, vx2 && vz2};
  int32_t lo = M[4], hi = M[4];
  bool big = false;
#pragma unroll
  for (int s9 = 0; s9 < 9; s9++) {
    const bool in = (s9 == 4) || val[s9 < 4 ? s9 : s9 - 1];
    const int32_t h = M[s9];
    if (in) {
      lo = min(lo, h);
      hi = max(hi, h);
      big |= (h < 0 ? -h : h) >= (1 << 27);
    }
  }
  const bool unit = kc.unit && !big && (long long)hi - (long long)lo < (1ll << 24);
  int it = 0;
  for (int r = 0; r < vis; r++) {
    const int tr = unit ? cascade_unit(M, val, kc.hd1, kc.hd2)
                        : (big ? cascade_general<long long>(M, val, kc, c) : cascade_general<int32_t>(M, val, kc, c));
    it++;
    if (tr == 0) break;
    st.transfers += tr;
  }
  st.cascades += it;
  st.cells += 1;
  if ((unsigned)it > st.max_iters) st.max_iters = (unsigned)it;
}

__device__ __forceinline__ CascadeConsts cascade_consts(const Consts& c) {
  CascadeConsts kc;
  kc.md1 = 1.0f * c.maxdiff;
  kc.md2 = kSqrt2 * c.maxdiff;
  kc.hd1 = kc.md1 * (0.5f * c.scale);
  kc.hd2 = kc.md2 * (0.5f * c.scale);
  kc.unit = c.settling == 1.0f;
  return kc;
}

// Colour phase: the owed cascades of every cell of colour (a, b).
//
// The 3x3 blocks around the colour-(0,0) cells tile the map (with virtual
// centres one step past the far edges), so the colour-0 phase first adds
// every cell's pending exchange delta, block by block: the same as adding
// all deltas before the first cascade.
//
// Each thread takes one cell and loads its 3x3 neighbourhood into its slice
// of shared memory; the cells that owe cascades are then compacted into a
// block-local list, and the block's threads work through that list densely,
// so warps are not held up by the threads whose cells owe nothing.
__device__ void colour_phase(const CycleArgs& A, int a, int b, int32_t* nb, int* list, int* owed, int* wcount,
                             CascadeStats& st) {
  const Consts& c = A.c;
  const int nx = c.nx, nz = c.nz;
  const bool absorb = (a == 0 && b == 0);
  const int cx = absorb ? nx / 3 + 1 : (nx - a + 2) / 3;
  const int cz = absorb ? nz / 3 + 1 : (nz - b + 2) / 3;
  const int cells = cx * cz;
  int32_t* H = A.B.hq;
  int32_t* Dq = A.B.dq;
  int32_t* V = A.B.visits;
  const CascadeConsts kc = cascade_consts(c);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  int32_t* N = nb + 9 * t;
  for (int base = blockIdx.x * blockDim.x; base < cells; base += gridDim.x * blockDim.x) {
    const int i = base + t;
    int visits = 0;
    if (i < cells) {
      const int ix = i / cz;
      const int x = a + 3 * ix, z = b + 3 * (i - ix * cz);
      const long g = (long)x * nz + z;
      if (x < nx && z < nz) {
        visits = V[g];
        if (visits) V[g] = 0;
      }
      if (absorb || visits) {
        bool changed = false;
#pragma unroll
        for (int u = 0; u < 3; u++) {
#pragma unroll
          for (int w = 0; w < 3; w++) {
            const bool ok = (u == 0 ? x > 0 : (u == 2 ? x + 1 < nx : x < nx)) &&
                            (w == 0 ? z > 0 : (w == 2 ? z + 1 < nz : z < nz));
            int32_t h = 0;
            if (ok) {
              const long q = g + (long)(u - 1) * nz + (w - 1);
              h = H[q];
              if (absorb) {
                const int32_t d = Dq[q];
                if (d != 0) {
                  h = wrap_add(h, d);
                  Dq[q] = 0;
                  changed = true;
                }
              }
            }
            N[3 * u + w] = h;
          }
        }
        if (changed && !visits) {
#pragma unroll
          for (int u = 0; u < 3; u++) {
#pragma unroll
            for (int w = 0; w < 3; w++) {
              const bool ok = (u == 0 ? x > 0 : (u == 2 ? x + 1 < nx : x < nx)) &&
                              (w == 0 ? z > 0 : (w == 2 ? z + 1 < nz : z < nz));
              if (ok) H[g + (long)(u - 1) * nz + (w - 1)] = N[3 * u + w];
            }
          }
        }
      }
    }
    // Compact the threads whose cell owes cascades.
    const unsigned m = __ballot_sync(0xffffffffu, visits != 0);
    if (lane == 0) wcount[warp] = __popc(m);
    owed[t] = visits;
    __syncthreads();
    int off = 0, total = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
      const int n = wcount[k];
      off += k < warp ? n : 0;
      total += n;
    }
    if (visits) list[off + __popc(m & ((1u << lane) - 1u))] = t;
    __syncthreads();
    if (t < total) {
      const int o = list[t];
      const int io = base + o;
      const int ix = io / cz;
      const int x = a + 3 * ix, z = b + 3 * (io - ix * cz);
      const long g = (long)x * nz + z;
      int32_t* M = nb + 9 * o;
      const int vis = owed[o];
      const bool vx0 = x > 0, vx2 = x + 1 < nx, vz0 = z > 0, vz2 = z + 1 < nz;
      cascade_cell(M, vx0, vx2, vz0, vz2, vis, kc, c, st);
#pragma unroll
      for (int u = 0; u < 3; u++) {
#pragma unroll
        for (int w = 0; w < 3; w++) {
          const bool ok = (u == 0 ? vx0 : (u == 2 ? vx2 : true)) && (w == 0 ? vz0 : (w == 2 ? vz2 : true));
          if (ok) H[g + (long)(u - 1) * nz + (w - 1)] = M[3 * u + w];
        }
      }
    }
    __syncthreads();
  }
}

// Tracks to float, EMA (world.hpp:70-76), heights to float, for cells
// i0, i0 + stride, ... With kWords the heights come from the cluster form's
// height words and are written back to the fixed-point map too.
template <bool kWords>
__device__ void ema_cells(const CycleArgs& A, long i0, long stride) {
  const long n = (long)A.c.nx * A.c.nz;
  unsigned bad = 0;
  const float lrate = A.c.lrate;
  for (long i = i0; i < n; i += stride) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float t = __ll2float_rn(A.B.tq[k][i]) * kInvTwo32;
      A.F.f[5 + k][i] = t;
      A.F.f[1 + k][i] = (1.0f - lrate) * A.F.f[1 + k][i] + lrate * t;
    }
    int32_t q;
    if constexpr (kWords) {
      q = (int32_t)(uint32_t)A.B.hw[i];
      A.B.hq[i] = q;
    } else {
      q = A.B.hq[i];
    }
    if (q > 1073741823 || q < -1073741823) bad = 1;
    A.F.f[0][i] = fx2f(q, A.c.inv_scale);
  }
  if (bad) atomicOr(&A.cnt->status, 0x2u);
}

__device__ void ema_phase(const CycleArgs& A) {
  ema_cells<false>(A, blockIdx.x * (long)blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x);
}

// Before a bounded-lanes cycle: height words with tag 0, owners none,
// visited bitmaps and track accumulators cleared, for cells i0, i0 + stride, ...
__device__ void prologue_cells(const ParallelBuffers& B, long n, long i0, long stride) {
  for (long i = i0; i < B.vbits_words; i += stride) {
    B.vbits[0][i] = 0;
    B.vbits[1][i] = 0;
    B.vbits[2][i] = 0;
  }
  for (long i = i0; i < n; i += stride) {
    B.hw[i] = (unsigned long long)(uint32_t)B.hq[i];
    B.owner[i] = 0x7FFFFFFF;
    B.owner2[i] = 0x7FFFFFFF;
    B.tq[0][i] = 0; B.tq[1][i] = 0; B.tq[2][i] = 0; B.tq[3][i] = 0;
  }
}

__global__ void __launch_bounds__(kCycleThreads, kCycleBlocksPerSm) k_par_cycle(CycleArgs A) {
  // Per-thread 3x3 neighbourhood of the colour phases (stride 9 words: the
  // 32 threads of a warp fall in distinct banks).
  __shared__ int32_t nb[kCycleThreads * 9];
  __shared__ int list[kCycleThreads];
  __shared__ int owed[kCycleThreads];
  __shared__ int wcount[kCycleThreads / 32];
  Counters* cnt = A.cnt;
  const unsigned long long cyc = cnt->cycle;
  const uint32_t c_lo = (uint32_t)cyc, c_hi = (uint32_t)(cyc >> 32);
  // Block 0's thread 0 times the phases (each including its closing barrier).
  const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long tph[13] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  unsigned long long t_mark = timer ? global_ns() : 0;
  auto lap = [&](int k) {
    if (timer) {
      const unsigned long long t = global_ns();
      tph[k] += t - t_mark;
      t_mark = t;
    }
  };

  spawn_phase(A, c_lo, c_hi);
  if (!grid_sync(A.gb, &cnt->status, wait_limit(A.c))) return;
  lap(0);

  CascadeStats cst;
  // Every step advances at least one particle, and each particle flies at
  // most max_age + 2 steps: a loop bound that is never reached.
  const long long max_steps = (long long)A.particles * (A.c.max_age + 2) + 2;
  for (long long step = 0; step < max_steps; step++) {
    const int in = (int)(step & 1), outp = in ^ 1;
    const int count = ld_volatile(&cnt->live[in]) + ld_volatile(&cnt->refill[in]);
    if (count == 0) break;
    fly_phase(A, in, count, c_lo, c_hi);
    if (!grid_sync(A.gb, &cnt->status, wait_limit(A.c))) return;
    lap(1);
    // Survivors and the particles that take the freed lanes; every block
    // reads the same counters here and computes the same refill.
    const int survivors = ld_volatile(&cnt->live[outp]);
    const int nid = ld_volatile(&cnt->next_id[in]);
    int refill = A.lanes - survivors;
    if (refill > A.particles - nid) refill = A.particles - nid;
    if (refill < 0) refill = 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      cnt->live[in] = 0;
      cnt->refill[outp] = refill;
      cnt->next_id[outp] = nid + refill;
    }
    if (survivors == 0) {
      // Only survivors wrote D and C: nothing to cascade.
      if (refill == 0) break;
      refill_lanes(A, outp, survivors, nid, refill, c_lo, c_hi);
      if (!grid_sync(A.gb, &cnt->status, wait_limit(A.c))) return;
      continue;
    }
    for (int col = 0; col < 9; col++) {
      if (col == 0) refill_lanes(A, outp, survivors, nid, refill, c_lo, c_hi);
      colour_phase(A, col / 3, col % 3, nb, list, owed, wcount, cst);
      if (!grid_sync(A.gb, &cnt->status, wait_limit(A.c))) return;
      lap(3 + col);
    }
  }
  {
    const unsigned long long tr = warp_sum(cst.transfers), ca = warp_sum(cst.cascades), ce = warp_sum(cst.cells);
    unsigned mi = cst.max_iters;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned other = __shfl_xor_sync(0xffffffffu, mi, o);
      mi = other > mi ? other : mi;
    }
    if ((threadIdx.x & 31) == 0) {
      if (tr) atomicAdd(&cnt->transfers, tr);
      if (ca) atomicAdd(&cnt->cascades, ca);
      if (ce) atomicAdd(&cnt->cascade_cells, ce);
      if (mi) atomicMax(&cnt->max_cascade_iters, mi);
    }
  }

  ema_phase(A);
  lap(12);
  if (timer) {
    cnt->cycle = cyc + 1;
    cnt->fly_ns += tph[1];
    unsigned long long cas = 0;
    for (int k = 3; k < 12; k++) cas += tph[k];
    cnt->cascade_ns += cas;
    for (int k = 0; k < 13; k++) cnt->phase_ns[k] += tph[k];
  }
}

// ---------------------------------------------------------------------------
// Bounded-lanes form of the cycle (k_par_lanes), for a bounded number of
// particles in flight.
//
// With few particles in flight a step is short, and the colour-phase
// kernel's eleven grid-wide barriers per step dominate it. Here each thread
// holds up to kClusterMaxSlots lanes (particle state in shared memory) and a
// step has one barrier: one 16-CTA thread-block cluster (hardware barrier,
// lane counts over distributed shared memory) for up to 4,096 lanes, else
// one CTA per SM of a cooperative grid (a flat barrier whose arrival atomic
// also sums the free lanes). A step:
//   fly      every particle flies against the heights the previous step left;
//            it adds one to its cell's visit count, marks the cell in the
//            step's visited bitmap and offers its lane id to the cell's owner
//            entry (atomicMin: the lowest id owns the cell), all without a
//            round trip;
//   barrier  every CTA learns the free lanes, and the cycle's next particles
//            take them (the same ids as in the colour-phase kernel: the set
//            of particles flying in a step is identical, only their lanes
//            differ);
//   cascade  each owner adds the cell's pending delta (H += D) and runs the
//            cell's owed cascades.
// The cascades are ordered cell by cell, reproducing the colour phases
// exactly: two cascades interact only if their 3x3 neighbourhoods overlap
// (cells at most 2 apart), and then the one of lower colour (x%3, z%3) runs
// first; every delta is added before any cascade reads the cell. Heights live
// here as 64-bit words, the fixed-point height in the low half and a tag in
// the high half: 16*(step+1) + the number of writes the cell has had in the
// step (its delta, then cascades). From the visited bits of the 5x5 cells
// around it, a cascade knows how many writes each cell of its 3x3 must have
// had before it reads it (the cell's own delta if it was visited, and the
// cascades of lower-colour visited cells next to it); it reads the words
// until their tags say so, then writes each cell back with its tag plus one.
// In the grid form the next step's flights check the tags of their five
// cells the same way (every write of the previous step), so no barrier
// separates a step's cascades from the next flights; the deltas, visit
// counts and owners of even and odd steps live in separate maps and the
// visited bitmaps rotate by step mod 3. In the cluster form a second
// hardware barrier ends every step instead.
// A value and its tag are written together by one 64-bit store, so the
// ordering rests on the coherence of single words alone: no memory fences
// (which serialise on an SM) are needed. Every wait is on a delta or on a
// lower colour, so the waits cannot form a cycle; a thread handles its cells
// in colour order, the polling loops are warp-uniform (a lane that is not
// ready polls again on the next pass, so it never holds up a lane of its own
// warp), and the CTAs are co-resident, so every wait ends. Each wait still
// has a deadline (2 s unless the world sets another): past it the thread sets SWE_STATUS_TIMEOUT and the
// abort flag, tagged with the barrier count, and every thread leaves the step
// loop after the same barrier.
// ---------------------------------------------------------------------------
constexpr int kClusterCtas = 16;
constexpr int kClusterMaxThreads = 256;  // up to 255 registers a thread
constexpr int kClusterMaxSlots = 4;
constexpr int kLanesGridMaxThreads = 256;
constexpr unsigned kClusterMaxSteps = 1u << 27;  // tags 16*(step+1)+k stay below 2^32

__device__ __forceinline__ void cluster_barrier() {
  // release/acquire at cluster scope (the defaults of arrive and wait)
  asm volatile("barrier.cluster.arrive;\n\tbarrier.cluster.wait;" ::: "memory");
}

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ unsigned cluster_ctas() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

// Reads a 32-bit word of CTA `rank`'s shared memory at the address of `p`.
__device__ __forceinline__ int ld_dsmem(const int* p, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  unsigned ra;
  int v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(ra) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}

__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v));
}

__device__ __forceinline__ int32_t word_height(unsigned long long w) { return (int32_t)(uint32_t)w; }
__device__ __forceinline__ unsigned word_tag(unsigned long long w) { return (unsigned)(w >> 32); }
__device__ __forceinline__ unsigned long long make_word(int32_t h, unsigned tag) {
  return ((unsigned long long)tag << 32) | (uint32_t)h;
}

// Whether a cell word's tag shows exactly `want` writes in the step whose
// tags start at `base` (want == 0: none, the tag is from an earlier step).
__device__ __forceinline__ bool tag_ready(unsigned tag, unsigned base, unsigned want) {
  return want ? tag == base + want : tag < base;
}

// Whether a thread gave up waiting before barrier number `ph` (the flag
// holds the count of barriers its writer had passed, plus one).
__device__ __forceinline__ bool aborted_before(GridBarrier* gb, unsigned ph) {
  const unsigned a = ld_acquire(&gb->abort);
  return a != 0 && a <= ph;
}

// Bit (du+2)*5 + (dw+2) for each cell of the 5x5 block around a cell; the
// cells next to (qu, qw) (itself included).
__host__ __device__ constexpr unsigned near_mask(int qu, int qw) {
  unsigned m = 0;
  for (int du = -2; du <= 2; du++)
    for (int dw = -2; dw <= 2; dw++)
      if (du - qu >= -1 && du - qu <= 1 && dw - qw >= -1 && dw - qw <= 1) m |= 1u << ((du + 2) * 5 + (dw + 2));
  return m;
}

// kCluster: the 16 CTAs of one cluster (cluster barriers, lane counts over
// distributed shared memory); otherwise one CTA per SM of a cooperative grid
// (grid barriers, lane counts in global memory).
// Visited bitmaps: cell i is bit 64 + i (64 bits of padding at both ends, so
// that the 5-bit runs read below never leave the array).
__device__ __forceinline__ void mark_visited(uint32_t* bm, long ci) {
  atomicOr(bm + ((ci + 64) >> 5), 1u << ((ci + 64) & 31));
}

// The visited bits of the 5x5 block around cell (x, z) (bit (du+2)*5 + dw+2),
// unmasked: rows off the map read the cell's own row, columns off the map
// read bits of the neighbouring rows; the caller masks both. The ten loads
// (load) and the assembly (bits) are split so that callers can issue other
// loads in between.
struct BlockBits {
  uint32_t lo[5], hi[5];
  unsigned sh[5];
  __device__ __forceinline__ void load(const uint32_t* bm, int x, int z, int nx, int nz) {
#pragma unroll
    for (int d = 0; d < 5; d++) {
      const int xr = (x + d - 2 >= 0 && x + d - 2 < nx) ? x + d - 2 : x;
      const long b = (long)xr * nz + z - 2 + 64;
      sh[d] = (unsigned)(b & 31);
      lo[d] = __ldcg(bm + (b >> 5));
      hi[d] = __ldcg(bm + (b >> 5) + 1);
    }
  }
  __device__ __forceinline__ unsigned bits() const {
    unsigned m = 0;
#pragma unroll
    for (int d = 0; d < 5; d++) m |= (__funnelshift_r(lo[d], hi[d], sh[d]) & 31u) << (5 * d);
    return m;
  }
};

template <bool kCluster>
__device__ __forceinline__ void lanes_cycle(const CycleArgs& A, int slots, int32_t* dyn) {
  __shared__ int s_free[2];            // free lanes of this CTA by step parity, read by the other CTAs
  __shared__ int s_all[kClusterCtas];  // every CTA's free lanes, this step (clusters of up to 16 CTAs)
  __shared__ int s_warp[32];
  // CTA 0's thread 0: flights + barrier, absorbs + cascades, last mark, tag
  // waits of the flights, barrier, refill + absorbs
  __shared__ unsigned long long s_time[6];
  const int T = blockDim.x;
  const int cap = slots * T;
  // Particle fields (id, age, sed_q, px, py, pz, vx, vy, vz) of lane slot j.
  auto PI = [&](int f, int j) -> int32_t& { return dyn[f * cap + j]; };
  auto PF = [&](int f, int j) -> float& { return reinterpret_cast<float*>(dyn)[f * cap + j]; };
  int* s_own = dyn + 9 * cap;        // per lane slot: the cell it owns this step
  int* s_vis = dyn + 10 * cap;       // per lane slot: cascades the owned cell owes
  int* s_ox = dyn + 11 * cap;        // per lane slot: the owned cell's x
  int32_t* N = dyn + 12 * cap + 9 * threadIdx.x;  // this thread's 3x3 neighbourhood
  // per lane slot and step parity: the cell the slot marked visited (-1: none)
  int* s_mark = dyn + 12 * cap + 9 * T;
  // Per cell colour (x%3, z%3): the cells of the 5x5 block around (bit
  // (du+2)*5 + dw+2) whose colour is lower.
  __shared__ unsigned s_lower[9];
  if (threadIdx.x < 9) {
    const int xr = threadIdx.x / 3, zr = threadIdx.x % 3;
    unsigned m = 0;
    for (int k = 0; k < 25; k++) {
      const int du = k / 5 - 2, dw = k % 5 - 2;
      if (((xr + du + 3) % 3) * 3 + (zr + dw + 3) % 3 < xr * 3 + zr) m |= 1u << k;
    }
    s_lower[threadIdx.x] = m;
  }
  __syncthreads();

  const Consts& c = A.c;
  const ParallelBuffers& B = A.B;
  unsigned long long* HW = B.hw;
  Counters* cnt = A.cnt;
  const int nx = c.nx, nz = c.nz;
  const unsigned r = kCluster ? cluster_rank() : blockIdx.x;
  const int nb = kCluster ? (int)cluster_ctas() : (int)gridDim.x;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5, nwarps = T >> 5;
  const unsigned long long cyc = cnt->cycle;
  const uint32_t c_lo = (uint32_t)cyc, c_hi = (uint32_t)(cyc >> 32);
  const CascadeConsts kc = cascade_consts(c);

  // This CTA's share of the lanes; slot s of thread t is lane slot s*T+t.
  const int L = A.lanes;
  const int Lr = L / nb + ((int)r < L % nb ? 1 : 0);
  unsigned lanes_mask = 0;
  const int order = A.spread ? lane * nwarps + warp : t;  // this thread's place in the CTA's lane order
#pragma unroll
  for (int s = 0; s < kClusterMaxSlots; s++)
    if (s < slots && s * T + order < Lr) lanes_mask |= 1u << s;
  unsigned live = 0;
  const int lane_id0 = (int)r * cap;  // lane slot j of this CTA has id lane_id0 + j

  const bool timer = r == 0 && t == 0;
  if (timer) {
    for (int k = 0; k < 6; k++) s_time[k] = 0;
    s_time[2] = global_ns();
  }
#pragma unroll
  for (int s = 0; s < kClusterMaxSlots; s++) {
    if (s < slots) {
      s_mark[2 * (s * T + t)] = -1;
      s_mark[2 * (s * T + t) + 1] = -1;
    }
  }

  unsigned ph = 0;  // barriers passed
  // 32-bit tallies, added to the counters before they could wrap
  CascadeTally<unsigned> cst;
  long long exported = 0;
  unsigned steps = 0;
  unsigned status = 0;
  bool gave_up = false;
  // Every step advances a particle, and each flies at most max_age + 2 steps:
  // a bound that is never reached (past it the cycle stops with
  // SWE_STATUS_TIMEOUT).
  const unsigned long long bound = (unsigned long long)A.particles * (c.max_age + 2) + 2;
  const unsigned max_steps = bound > kClusterMaxSteps ? kClusterMaxSteps : (unsigned)bound;

  // The cycle's particles with ids from `first` take the free lanes `freem`
  // of this thread; `rank` is the CTA-wide rank of its first free lane among
  // all free lanes, and `count` lanes in all are filled.
  auto spawn = [&](unsigned freem, int rank, int first, int count) {
#pragma unroll
    for (int s = 0; s < kClusterMaxSlots; s++) {
      if ((freem >> s) & 1u) {
        if (rank < count) {
          const int id = first + rank;
          const uint4 u = philox4x32((uint32_t)id, 0xFFFFFFFFu, c_lo, c_hi, A.seed_lo, A.seed_hi);
          const int j = s * T + t;
          PI(0, j) = id;
          PI(1, j) = 0;
          PI(2, j) = 0;
          PF(3, j) = (float)(int)(u.x % (uint32_t)nx) + (float)(int)(u.z % 1000u) / 1000.0f;
          PF(4, j) = 0.0f;
          PF(5, j) = (float)(int)(u.y % (uint32_t)nz) + (float)(int)(u.w % 1000u) / 1000.0f;
          PF(6, j) = 0.0f; PF(7, j) = 0.0f; PF(8, j) = 0.0f;
          live |= 1u << s;
        }
        rank++;
      }
    }
  };
  // CTA-wide exclusive prefix of the threads' counts f (and the CTA total).
  auto block_scan = [&](int f, int* total) -> int {
    int incl = f;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    __syncthreads();  // s_warp is free again
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    int wpre = 0, tot = 0;
    for (int k = 0; k < nwarps; k++) {
      const int v = s_warp[k];
      wpre += k < warp ? v : 0;
      tot += v;
    }
    *total = tot;
    return wpre + incl - f;
  };

  // The first lanes of the cycle: every lane free, ids in lane order.
  int nid;
  {
    int btotal = 0;
    const int pre = block_scan(__popc(lanes_mask), &btotal);
    const int base0 = (int)r * (L / nb) + ((int)r < L % nb ? (int)r : L % nb);
    nid = A.particles < L ? A.particles : L;
    spawn(lanes_mask, base0 + pre, 0, nid);
  }

  // One step: every particle flies once its five cells have had every write
  // of the previous step (the tags of their words say so); one barrier, at
  // which the free lanes are counted; the next particles take the free lanes;
  // the owned cells absorb their deltas and run their cascades. A thread goes
  // on to its next flight as soon as its own cascades are done: the deltas,
  // visit counts and owners of consecutive steps live in separate maps.
  unsigned rot = 0;  // step mod 3
  for (unsigned step = 0;; step++, rot = rot == 2 ? 0 : rot + 1) {
    if (cst.transfers > 0x40000000u || cst.cascades > 0x40000000u || steps > 0x40000000u) {
      atomicAdd(&cnt->transfers, (unsigned long long)cst.transfers);
      atomicAdd(&cnt->cascades, (unsigned long long)cst.cascades);
      atomicAdd(&cnt->particle_steps, (unsigned long long)steps);
      cst.transfers = 0;
      cst.cascades = 0;
      steps = 0;
    }
    const unsigned odd = step & 1u;
    const unsigned tbase = 16u * (step + 1);  // tag base of this step
    // visited bitmaps by step mod 3: this step's, the previous step's, and
    // the one two steps back, cleared now (its last readers were the
    // previous step's flights; its next writers fly after this step's
    // barrier): every lane slot clears the word of the cell it marked then,
    // so every set bit is cleared, word by word
    uint32_t* vb = B.vbits[rot];
    const uint32_t* vb_prev = B.vbits[rot == 0 ? 2 : rot - 1];
    {
      uint32_t* vb_clear = B.vbits[rot == 2 ? 0 : rot + 1];
#pragma unroll
      for (int s = 0; s < kClusterMaxSlots; s++) {
        if (s < slots) {
          const int m = s_mark[2 * (s * T + t) + (step & 1u)];
          if (m >= 0) vb_clear[((long)m + 64) >> 5] = 0u;
          s_mark[2 * (s * T + t) + (step & 1u)] = -1;
        }
      }
    }
    int32_t* visits = odd ? B.visits2 : B.visits;
    int32_t* dq = odd ? B.dq2 : B.dq;
    int32_t* owner = odd ? B.owner2 : B.owner;

    // Fly.
    unsigned flew = 0;  // bit s: slot s flew this step (its cell is in s_own)
#pragma unroll
    for (int s = 0; s < kClusterMaxSlots; s++) {
      if (s >= slots) break;
      const int j = s * T + t;
      Particle p;
      long ci = -1;
      int ix = 0, iz = 0;
      if ((live >> s) & 1u) {
        p.id = PI(0, j); p.age = PI(1, j); p.sed_q = PI(2, j);
        p.px = PF(3, j); p.py = PF(4, j); p.pz = PF(5, j);
        p.vx = PF(6, j); p.vy = PF(7, j); p.vz = PF(8, j);
        ci = particle_cell(c, p, ix, iz);
      }
      // The five cells' words (bits 0..4: the cell, x-1, x+1, z-1, z+1),
      // each read until its tag shows every write of the previous step: the
      // cell's delta if it was visited, and the cascades of the visited cells
      // next to it (from the previous step's visited bits of the 5x5 block).
      const long nbr[5] = {0, -(long)nz, (long)nz, -1, 1};
      const int qpos[5] = {12, 7, 17, 11, 13};  // positions in the 5x5 block
      unsigned need = 0, ready = 0, prev = 0, inm = 0, fwant = 0;
      int32_t hv[5] = {0, 0, 0, 0, 0};
      BlockBits pb;
      // (In a cluster a second barrier ends every step instead, so every
      // word is final here and no tag is checked.)
      const bool check = !kCluster && step > 0;
      if (ci >= 0) {
        need = 1u | (ix > 0 ? 2u : 0u) | (ix + 1 < nx ? 4u : 0u) | (iz > 0 ? 8u : 0u) | (iz + 1 < nz ? 16u : 0u);
        if (check) {
          unsigned rows = 0, cols = 0;
#pragma unroll
          for (int d = -2; d <= 2; d++) {
            rows |= (ix + d >= 0 && ix + d < nx) ? 1u << (d + 2) : 0u;
            cols |= (iz + d >= 0 && iz + d < nz) ? 1u << (d + 2) : 0u;
          }
#pragma unroll
          for (int d = 0; d < 5; d++) inm |= ((rows >> d) & 1u) ? cols << (5 * d) : 0u;
          pb.load(vb_prev, ix, iz, nx, nz);
        }
      }
      const unsigned pbase = 16u * step;  // tag base of the previous step
      unsigned long long t_wait = 0;
      Turbulence tb{0.0f, 0.0f, 0.0f};
      for (bool first = true;; first = false) {
        // five loads every pass (rows off the map read the cell's own row;
        // columns off the map land in the padding word or the next row)
        unsigned long long wd[5] = {0, 0, 0, 0, 0};
        if (ci >= 0) {
#pragma unroll
          for (int q = 0; q < 5; q++) wd[q] = ld_relaxed64(HW + ci + ((need >> q) & 1u ? nbr[q] : 0));
        }
        // the step's turbulence draws need no height: taken while the loads fly
        if (first && ci >= 0) tb = turbulence(p, c_lo, c_hi, A.seed_lo, A.seed_hi);
        if (first && check && ci >= 0) {
          prev = pb.bits() & inm;
#pragma unroll
          for (int q = 0; q < 5; q++) {
            const int qu = qpos[q] / 5 - 2, qw = qpos[q] % 5 - 2;
            fwant |= (__popc(prev & near_mask(qu, qw)) + ((prev >> qpos[q]) & 1u)) << (4 * q);
          }
        }
#pragma unroll
        for (int q = 0; q < 5; q++) {
          if (((need & ~ready) >> q) & 1u) {
            const unsigned want = (fwant >> (4 * q)) & 15u;
            if (!check || tag_ready(word_tag(wd[q]), pbase, want)) {
              hv[q] = word_height(wd[q]);
              ready |= 1u << q;
            }
          }
        }
        if (ready != need && !gave_up) {
          const unsigned long long now = global_ns();
          if (t_wait == 0) t_wait = now;
          if (now - t_wait > wait_limit(c) || ld_volatile(reinterpret_cast<const int*>(&A.gb->abort)) != 0) {
            status |= 0x8u;  // SWE_STATUS_TIMEOUT
            atomicCAS(&A.gb->abort, 0u, ph + 1);
            gave_up = true;
          }
        }
        if (gave_up) ready = need;
        if (!__any_sync(0xffffffffu, ready != need)) break;
        __nanosleep(64);
      }
      if (timer) {
        const unsigned long long now = global_ns();
        s_time[0] += now - s_time[2];
        s_time[3] += now - s_time[2];
        s_time[2] = now;
      }
      if ((live >> s) & 1u) {
        if (ci >= 0 && !gave_up)
          ci = fly_from(c, B, dq, ci, ix, iz, hv[0], hv[1], hv[2], hv[3], hv[4], tb, p, status);
        else
          ci = -1;
        if (ci >= 0) {
          steps++;
          // One cascade owed to the cell; the lowest lane id among the
          // cell's visitors becomes its owner (both without a round trip).
          atomicAdd(visits + ci, 1);
          atomicMin(owner + ci, lane_id0 + j);
          mark_visited(vb, ci);
          s_mark[2 * j + (step & 1u)] = (int)ci;
          s_own[j] = (int)ci;
          s_ox[j] = ix;
          flew |= 1u << s;
          PI(1, j) = p.age; PI(2, j) = p.sed_q;
          PF(3, j) = p.px; PF(4, j) = p.py; PF(5, j) = p.pz;
          PF(6, j) = p.vx; PF(7, j) = p.vy; PF(8, j) = p.vz;
        } else {
          exported += p.sed_q;
          live &= ~(1u << s);
        }
      }
    }

    // The step's one barrier: every exchange and visit of the step is in,
    // and the free lanes are counted on the way.
    if (timer) {
      const unsigned long long now = global_ns();
      s_time[0] += now - s_time[2];
      s_time[2] = now;
    }
    const unsigned freem = lanes_mask & ~live;
    int btotal = 0;
    const int pre = block_scan(__popc(freem), &btotal);
    int total_free = 0, base = 0;
    if constexpr (kCluster) {
      if (t == 0) s_free[odd] = btotal;
      cluster_barrier();
      ph++;
      if (aborted_before(A.gb, ph)) break;
      if (t < nb) s_all[t] = ld_dsmem(&s_free[odd], (unsigned)t);
      __syncthreads();
      for (int k = 0; k < nb; k++) {
        const int v = s_all[k];
        total_free += v;
        base += k < (int)r ? v : 0;
      }
    } else {
      unsigned below = 0, tot = 0;
      if (!grid_sync_sum(A.gb, &cnt->status, wait_limit(c), rot, (unsigned)btotal, &below, &tot)) break;
      ph++;
      total_free = (int)tot;
      base = (int)below;
    }
    if (timer) {
      const unsigned long long now = global_ns();
      s_time[0] += now - s_time[2];
      s_time[4] += now - s_time[2];
      s_time[2] = now;
    }
    const int survivors = L - total_free;
    int refill = A.particles - nid;
    if (refill > total_free) refill = total_free;
    // Nobody flew (no survivors, so no writes) and nobody is left: done.
    const bool done = (survivors == 0 && refill == 0) || step + 1 >= max_steps;
    if (step + 1 >= max_steps && !(survivors == 0 && refill == 0)) status |= 0x8u;  // SWE_STATUS_TIMEOUT
    if (!done) {
      spawn(freem, base + pre, nid, refill);
      nid += refill;
    }

    // Owners and their cells' deltas: the first write of each cell in the
    // step, before any cascade waits. Every lane that flew loads its cell's
    // owner, visit, delta and word entries in one batch; the owner clears the
    // owner, visit and delta entries (a visitor reading the owner entry after
    // that sees no match either).
    unsigned owned = 0;
#pragma unroll
    for (int s = 0; s < kClusterMaxSlots; s++) {
      if ((flew >> s) & 1u) {
        const int ci = s_own[s * T + t];
        const int ow = __ldcg(owner + ci);
        const int v = __ldcg(visits + ci);
        const int32_t d = __ldcg(dq + ci);
        const unsigned long long w = ld_relaxed64(HW + ci);
        if (ow == lane_id0 + s * T + t) {
          owned |= 1u << s;
          s_vis[s * T + t] = v;
          __stcg(visits + ci, 0);
          __stcg(dq + ci, 0);
          __stcg(owner + ci, 0x7FFFFFFF);
          st_relaxed64(HW + ci, make_word(wrap_add(word_height(w), d), tbase + 1));
        }
      }
    }
    if (timer) {
      const unsigned long long now = global_ns();
      s_time[1] += now - s_time[2];
      s_time[5] += now - s_time[2];
      s_time[2] = now;
    }
    // Cascades of the owned cells. Each lane takes its cells in colour order
    // (lowest first) and cascades one as soon as the tags of its 3x3 words
    // show every earlier write. The loop is warp-uniform: a lane whose cell
    // is not ready yet polls again on the next pass instead of spinning, so
    // a lane waiting for another lane of its own warp never holds that lane
    // up. Every pass issues its loads in one batch.
    {
      unsigned todo = owned;  // slots whose cell still owes its cascades
      int cs = -1;            // slot of the cell in hand
      int ci = 0, x = 0, z = 0;
      unsigned visited = 0, lower = 0, ready = 0, okmask = 0, inmask = 0;
      unsigned long long wants = 0;  // 4 bits per word of the 3x3: the writes it must have had
      unsigned long long t_wait = 0;
      // the 3x3 words by row (rows off the map point at the cell's own row,
      // columns off the map land in the padding word or the next row)
      unsigned long long* rp[3] = {HW, HW, HW};
      for (;;) {
        bool progressed = false;
        bool fresh = false;  // a new cell in hand: its visited bits were loaded in this pass
        BlockBits cb;
        if (cs < 0 && todo && !gave_up) {
          // the lowest-colour cell left
          if (slots == 1) {
            cs = 0;
          } else {
            int best = 9;
#pragma unroll
            for (int s2 = 0; s2 < kClusterMaxSlots; s2++) {
              if ((todo >> s2) & 1u) {
                const int x2 = s_ox[s2 * T + t], z2 = s_own[s2 * T + t] - x2 * nz;
                const int col2 = (x2 % 3) * 3 + z2 % 3;
                if (col2 < best) {
                  best = col2;
                  cs = s2;
                }
              }
            }
          }
          ci = s_own[cs * T + t];
          x = s_ox[cs * T + t];
          z = ci - x * nz;
          // In-map rows and columns of the 5x5 block, as bit masks.
          unsigned rows = 0, cols = 0;
#pragma unroll
          for (int d = -2; d <= 2; d++) {
            rows |= (x + d >= 0 && x + d < nx) ? 1u << (d + 2) : 0u;
            cols |= (z + d >= 0 && z + d < nz) ? 1u << (d + 2) : 0u;
          }
          inmask = 0;
#pragma unroll
          for (int d = 0; d < 5; d++) inmask |= ((rows >> d) & 1u) ? cols << (5 * d) : 0u;
          // visited bits of the 5x5 block around (assembled below)
          cb.load(vb, x, z, nx, nz);
          rp[1] = HW + ci - 1;
          rp[0] = x > 0 ? rp[1] - nz : rp[1];
          rp[2] = x + 1 < nx ? rp[1] + nz : rp[1];
          // the 3x3 neighbourhood's in-map cells (bit 3u+w)
          okmask = 0;
#pragma unroll
          for (int u = 0; u < 3; u++)
#pragma unroll
            for (int w = 0; w < 3; w++) okmask |= ((inmask >> ((u + 1) * 5 + w + 1)) & 1u) << (3 * u + w);
          ready = 0;
          t_wait = 0;
          fresh = true;
        }
        // The words not taken yet, loaded in the same batch as the visited bits
        // (taken or off-map words read the cell's own word and are masked).
        unsigned long long wd[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (cs >= 0) {
#pragma unroll
          for (int q = 0; q < 9; q++) wd[q] = ld_relaxed64(rp[q / 3] + q % 3);
        }
        if (fresh) {
          // visited cells of the 5x5 block, and those of lower colour
          visited = (cb.bits() & inmask) | (1u << 12);
          lower = visited & s_lower[(x % 3) * 3 + z % 3];
          wants = 0;
#pragma unroll
          for (int q = 0; q < 9; q++) {
            const int u = q / 3, w = q % 3;
            const unsigned want = __popc(lower & near_mask(u - 1, w - 1)) + ((visited >> ((u + 1) * 5 + w + 1)) & 1u);
            wants |= (unsigned long long)want << (4 * q);
          }
        }

        if (cs >= 0) {
          // Take the words whose tags show every earlier write (the cell's
          // own delta if visited, the cascades of the lower-colour visited
          // cells next to it).
#pragma unroll
          for (int q = 0; q < 9; q++) {
            const bool need = ((okmask & ~ready) >> q) & 1u;
            const unsigned want = (unsigned)(wants >> (4 * q)) & 15u;
            if (need && tag_ready(word_tag(wd[q]), tbase, want)) {
              N[q] = word_height(wd[q]);
              ready |= 1u << q;
            }
          }
          if (ready == okmask) {
            cascade_cell(N, x > 0, x + 1 < nx, z > 0, z + 1 < nz, s_vis[cs * T + t], kc, c, cst);
            // Every cell of the neighbourhood takes its next tag, changed or not.
#pragma unroll
            for (int q = 0; q < 9; q++) {
              if ((okmask >> q) & 1u) {
                const unsigned want = (unsigned)(wants >> (4 * q)) & 15u;
                st_relaxed64(rp[q / 3] + q % 3, make_word(N[q], tbase + want + 1));
              }
            }
            todo &= ~(1u << cs);
            cs = -1;
            progressed = true;
          } else {
            // Not ready: a deadline, and the abort flag of another thread.
            const unsigned long long now = global_ns();
            if (t_wait == 0) t_wait = now;
            if (now - t_wait > wait_limit(c) || ld_volatile(reinterpret_cast<const int*>(&A.gb->abort)) != 0) {
              if (!gave_up) {
                status |= 0x8u;  // SWE_STATUS_TIMEOUT
                atomicCAS(&A.gb->abort, 0u, ph + 1);
              }
              gave_up = true;
              cs = -1;
              todo = 0;
            }
          }
        }
        const bool more = cs >= 0 || (todo != 0 && !gave_up);
        if (!__any_sync(0xffffffffu, more)) break;
        if (!__any_sync(0xffffffffu, progressed)) __nanosleep(64);
      }
    }
    if constexpr (kCluster) {
      // the cheap hardware barrier makes every write of the step visible
      // before the next flights (instead of checking tags in them)
      cluster_barrier();
      ph++;
    }
    if (timer) {
      const unsigned long long now = global_ns();
      s_time[1] += now - s_time[2];
      s_time[2] = now;
    }
    if (done) break;
    if constexpr (kCluster) {
      if (aborted_before(A.gb, ph)) break;
    }
  }
  // No CTA may leave while another can still read its shared memory.
  if constexpr (kCluster) cluster_barrier();

  // Tallies.
  {
    const unsigned long long tr = warp_sum((unsigned long long)cst.transfers);
    const unsigned long long ca = warp_sum((unsigned long long)cst.cascades);
    const unsigned long long ce = warp_sum((unsigned long long)cst.cells);
    const long long ex = warp_sum(exported);
    const unsigned long long stp = warp_sum((unsigned long long)steps);
    const unsigned stt = __reduce_or_sync(0xffffffffu, status);
    unsigned mi = cst.max_iters;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned other = __shfl_xor_sync(0xffffffffu, mi, o);
      mi = other > mi ? other : mi;
    }
    if (lane == 0) {
      if (tr) atomicAdd(&cnt->transfers, tr);
      if (ca) atomicAdd(&cnt->cascades, ca);
      if (ce) atomicAdd(&cnt->cascade_cells, ce);
      if (mi) atomicMax(&cnt->max_cascade_iters, mi);
      if (ex) atomicAdd((unsigned long long*)&cnt->exported_q, (unsigned long long)ex);
      if (stp) atomicAdd(&cnt->particle_steps, stp);
      if (stt) atomicOr(&cnt->status, stt);
    }
  }
  if (timer) {
    cnt->cycle = cyc + 1;
    cnt->particles += (unsigned long long)A.particles;
    cnt->fly_ns += s_time[0];
    cnt->cascade_ns += s_time[1];
    cnt->phase_ns[1] += s_time[0];
    cnt->phase_ns[3] += s_time[1];
    cnt->phase_ns[0] += s_time[3];
    cnt->phase_ns[2] += s_time[4];
    cnt->phase_ns[4] += s_time[5];
  }
}

template <bool kCluster>
__global__ void __launch_bounds__(kCluster ? kClusterMaxThreads : kLanesGridMaxThreads, 1)
    k_par_lanes(CycleArgs A, int slots) {
  extern __shared__ int32_t dyn[];
  lanes_cycle<kCluster>(A, slots, dyn);
}

// An ensemble of independent worlds in one persistent launch: each 16-CTA
// cluster takes the next world from a queue and runs all of its cycles
// (the map sweeps by the cluster's own threads, the steps as above), so
// every world's result is the one a launch of its own would give.
struct BatchItem {
  CycleArgs A;
  int slots;
  int pad;
};

__global__ void __launch_bounds__(kClusterMaxThreads, 1)
    k_par_batch(const BatchItem* __restrict__ items, int count, int cycles, unsigned* queue) {
  extern __shared__ int32_t dyn[];
  __shared__ int s_item;
  __shared__ CycleArgs s_args;
  __shared__ int s_slots;
  const unsigned r = cluster_rank();
  const int T = blockDim.x;
  const long tid = (long)r * T + threadIdx.x, nthr = (long)cluster_ctas() * T;
  for (;;) {
    if (r == 0 && threadIdx.x == 0) s_item = (int)atomicAdd(queue, 1u);
    cluster_barrier();
    const int item = ld_dsmem(&s_item, 0);
    cluster_barrier();  // CTA 0 keeps its shared memory until every CTA has read it
    if (item >= count) break;
    // This world's arguments, copied to shared memory word by word.
    {
      const int* src = reinterpret_cast<const int*>(&items[item].A);
      int* dst = reinterpret_cast<int*>(&s_args);
      for (int k = threadIdx.x; k < (int)(sizeof(CycleArgs) / sizeof(int)); k += T) dst[k] = src[k];
      if (threadIdx.x == 0) s_slots = items[item].slots;
    }
    __syncthreads();
    const CycleArgs& A = s_args;
    const long n = (long)A.c.nx * A.c.nz;
    for (int k = 0; k < cycles; k++) {
      if (r == 0 && threadIdx.x == 0) A.gb->abort = 0;
      prologue_cells(A.B, n, tid, nthr);
      cluster_barrier();
      lanes_cycle<true>(A, s_slots, dyn);  // ends with a cluster barrier
      ema_cells<true>(A, tid, nthr);         // the same cells per thread as the prologue
    }
    cluster_barrier();
  }
}

// The sweeps around a bounded-lanes cycle, on the whole GPU.
__global__ void k_cluster_prologue(ParallelBuffers B, long n) {
  prologue_cells(B, n, blockIdx.x * (long)blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x);
}

__global__ void k_ema_cycle(CycleArgs A) {
  ema_cells<true>(A, blockIdx.x * (long)blockDim.x + threadIdx.x, (long)gridDim.x * blockDim.x);
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

int cycle_grid(int device) {
  int sms = 0, per_sm = 0, coop = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_par_cycle, kCycleThreads, 0) != cudaSuccess)
    return 0;
  return sms * per_sm;
}

int par_lanes(int lanes, int nx, int nz, int particles) {
  long l;
  if (lanes > 0) {
    l = lanes;
  } else if (lanes == 0) {
    l = (long)nx * nz / 256;
    if (l < 1024) l = 1024;
  } else {
    l = particles;
  }
  if (l > particles) l = particles;
  return (int)(l < 1 ? 1 : l);
}

namespace {

// Bounded-lanes launch shapes. One cluster (16 CTAs) takes up to
// kClusterMaxLanes lanes; beyond that one CTA per SM of a cooperative grid.
// Threads per CTA are a multiple of 32 up to 256, with up to
// kClusterMaxSlots lanes per thread.
constexpr int kClusterMaxLanes = 4096;

bool lanes_shape(int lanes, int ctas, int max_threads, int* threads, int* slots) {
  const int per_cta = (lanes + ctas - 1) / ctas;
  int t = (per_cta + 31) / 32 * 32;
  if (t > max_threads) t = max_threads;
  const int k = (per_cta + t - 1) / t;
  if (k > kClusterMaxSlots) return false;
  *threads = t;
  *slots = k;
  return true;
}

// particle state (9 words), owned cell, owed cascades, the cell's x and the
// cells marked visited in the last two steps (5 words) per lane slot, and a
// 3x3 neighbourhood per thread
size_t lanes_smem(int threads, int slots) { return sizeof(int32_t) * (size_t)threads * (14 * slots + 9); }

cudaError_t launch_cluster(const CycleArgs& A, int threads, int slots, cudaStream_t s, bool* launched) {
  *launched = false;
  const size_t smem = lanes_smem(threads, slots);
  cudaError_t e = cudaFuncSetAttribute(k_par_lanes<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_par_lanes<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cudaSuccess;  // not available: the caller takes another form
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kClusterCtas);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kClusterCtas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, k_par_lanes<true>, &cfg) != cudaSuccess || clusters < 1) {
    cudaGetLastError();
    return cudaSuccess;
  }
  e = cudaLaunchKernelEx(&cfg, k_par_lanes<true>, A, slots);
  *launched = e == cudaSuccess;
  return e;
}

int sms_of_current() {
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

cudaError_t launch_lanes_grid(const CycleArgs& A, int ctas, int threads, int slots, cudaStream_t s,
                              bool* launched) {
  *launched = false;
  const size_t smem = lanes_smem(threads, slots);
  cudaError_t e = cudaFuncSetAttribute(k_par_lanes<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per_sm = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_par_lanes<false>, threads, smem);
  if (e != cudaSuccess || per_sm < 1 || ctas > per_sm * sms_of_current()) {
    cudaGetLastError();
    return cudaSuccess;  // not co-resident: the caller takes another form
  }
  int sl = slots;
  void* args[] = {const_cast<CycleArgs*>(&A), &sl};
  e = cudaLaunchCooperativeKernel((const void*)k_par_lanes<false>, dim3(ctas), dim3(threads), args, smem, s);
  *launched = e == cudaSuccess;
  return e;
}

}  // namespace

cudaError_t launch_par_cycle(const ParallelBuffers& B, const Fields& F, const Consts& c, uint64_t seed,
                             Counters* cnt, GridBarrier* gb, int particles, int lanes, int grid, cudaStream_t s,
                             const LaunchForm& form) {
  CycleArgs A;
  A.B = B;
  A.F = F;
  A.c = c;
  A.seed_lo = (uint32_t)seed;
  A.seed_hi = (uint32_t)(seed >> 32);
  A.cnt = cnt;
  A.gb = gb;
  A.particles = particles;
  A.lanes = lanes;
  A.spread = 0;
  const long n = (long)c.nx * c.nz;
  // Bounded lanes: one cluster, or one CTA per SM; cell indices are 32-bit there.
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms > 1024) sms = 1024;
  int threads = 0, slots = 0;
  // The form: by default one cluster up to kClusterMaxLanes lanes, else one
  // CTA per SM; a requested form that cannot hold the lanes takes the default.
  bool cluster = lanes <= kClusterMaxLanes;
  int ctas = sms;
  if (form.kind == 1 && lanes_shape(lanes, kClusterCtas, kClusterMaxThreads, &threads, &slots)) {
    cluster = true;
  } else if (form.kind == 2 || form.kind == 3) {
    const int want = form.ctas > 0 && form.ctas <= 4 * sms ? form.ctas : sms;
    if (lanes_shape(lanes, want, kLanesGridMaxThreads, &threads, &slots)) {
      cluster = false;
      ctas = want;
      A.spread = form.kind == 3 ? 1 : 0;
    }
  }
  if (n <= (1l << 30) && lanes_shape(lanes, cluster ? kClusterCtas : ctas,
                                     cluster ? kClusterMaxThreads : kLanesGridMaxThreads, &threads, &slots)) {
    if (A.spread && threads < 128) {
      // four warps share the CTA's lanes (at most 96 of them here: one slot each)
      threads = 128;
      slots = 1;
    }
    k_cluster_prologue<<<sweep_grid(n), 256, 0, s>>>(B, n);
    bool launched = false;
    const cudaError_t e = cluster ? launch_cluster(A, threads, slots, s, &launched)
                                  : launch_lanes_grid(A, ctas, threads, slots, s, &launched);
    if (e != cudaSuccess) return e;
    if (launched) {
      k_ema_cycle<<<sweep_grid(n), 256, 0, s>>>(A);
      return cudaGetLastError();
    }
  }
  // All particles at once: the particle state lives in B.state.
  if (B.capacity < lanes || !B.state[0].id) return cudaErrorInvalidValue;
  void* args[] = {&A};
  return cudaLaunchCooperativeKernel((const void*)k_par_cycle, dim3(grid), dim3(kCycleThreads), args, 0, s);
}

bool lanes_form_fits(int lanes, long n) {
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms > 1024) sms = 1024;
  int threads = 0, slots = 0;
  const bool cluster = lanes <= kClusterMaxLanes;
  return n <= (1l << 30) && lanes_shape(lanes, cluster ? kClusterCtas : sms,
                                        cluster ? kClusterMaxThreads : kLanesGridMaxThreads, &threads, &slots);
}

__global__ void k_set_cycle(Counters* cnt, unsigned long long cycle) { cnt->cycle = cycle; }

void launch_set_cycle(Counters* cnt, uint64_t cycle, cudaStream_t s) { k_set_cycle<<<1, 1, 0, s>>>(cnt, cycle); }

bool batch_fits(int lanes, int nx, int nz) {
  int threads = 0, slots = 0;
  return (long)nx * nz <= (1l << 30) &&
         lanes_shape(lanes, kClusterCtas, kClusterMaxThreads, &threads, &slots);
}

bool batch_shape_ok(const BatchShape& sh) {
  return (sh.ctas == 4 || sh.ctas == 8 || sh.ctas == 16) && sh.threads >= 32 && sh.threads <= kClusterMaxThreads &&
         sh.threads % 32 == 0;
}

size_t batch_item_bytes() { return sizeof(BatchItem); }

cudaError_t upload_batch_items(const BatchWorld* worlds, int count, const BatchShape& sh, void* d_items,
                               cudaStream_t s) {
  if (!batch_shape_ok(sh)) return cudaErrorInvalidValue;
  // Largest worlds first (cells x particles), so that the last clusters to
  // finish are not the ones that started the longest worlds last.
  std::vector<int> order((size_t)count);
  for (int i = 0; i < count; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const double wa = (double)worlds[a].c.nx * worlds[a].c.nz * worlds[a].particles;
    const double wb = (double)worlds[b].c.nx * worlds[b].c.nz * worlds[b].particles;
    return wa > wb;
  });
  std::vector<BatchItem> items((size_t)count);
  for (int i = 0; i < count; i++) {
    const BatchWorld& w = worlds[order[i]];
    CycleArgs& A = items[i].A;
    A.B = w.B;
    A.F = w.F;
    A.c = w.c;
    A.seed_lo = (uint32_t)w.seed;
    A.seed_hi = (uint32_t)(w.seed >> 32);
    A.cnt = w.cnt;
    A.gb = w.gb;
    A.particles = w.particles;
    A.lanes = w.lanes;
    A.spread = 0;
    int threads = 0, slots = 0;
    if ((long)w.c.nx * w.c.nz > (1l << 30) || !lanes_shape(w.lanes, sh.ctas, sh.threads, &threads, &slots))
      return cudaErrorInvalidValue;
    items[i].slots = slots;
    items[i].pad = 0;
  }
  cudaError_t e = cudaMemcpyAsync(d_items, items.data(), sizeof(BatchItem) * (size_t)count, cudaMemcpyHostToDevice, s);
  // the host array must outlive the copy
  const cudaError_t es = cudaStreamSynchronize(s);
  return e != cudaSuccess ? e : es;
}

namespace {

void batch_launch_config(const BatchShape& sh, int clusters, cudaStream_t s, cudaLaunchConfig_t* cfg,
                         cudaLaunchAttribute* attr) {
  *cfg = cudaLaunchConfig_t{};
  cfg->gridDim = dim3(sh.ctas * clusters);
  cfg->blockDim = dim3(sh.threads);
  cfg->dynamicSmemBytes = lanes_smem(sh.threads, kClusterMaxSlots);
  cfg->stream = s;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = sh.ctas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg->attrs = attr;
  cfg->numAttrs = 1;
}

}  // namespace

int batch_clusters(const BatchShape& sh, int count) {
  if (!batch_shape_ok(sh) || count < 1) return 0;
  // the largest shared-memory size any shape asks for
  const size_t smem = lanes_smem(kClusterMaxThreads, kClusterMaxSlots);
  cudaError_t e = cudaFuncSetAttribute(k_par_batch, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_par_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr[1];
  batch_launch_config(sh, 1, nullptr, &cfg, attr);
  int clusters = 0;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&clusters, k_par_batch, &cfg);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return clusters < count ? clusters : count;
}

cudaError_t launch_batch_items(const void* d_items, unsigned* d_queue, int count, int cycles, const BatchShape& sh,
                               int clusters, cudaStream_t s) {
  if (count <= 0 || cycles <= 0) return cudaSuccess;
  if (!batch_shape_ok(sh) || clusters < 1) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr[1];
  batch_launch_config(sh, clusters, s, &cfg, attr);
  cudaError_t e = cudaMemsetAsync(d_queue, 0, sizeof(unsigned), s);
  if (e == cudaSuccess)
    e = cudaLaunchKernelEx(&cfg, k_par_batch, static_cast<const BatchItem*>(d_items), count, cycles, d_queue);
  return e;
}

cudaError_t launch_par_batch(const BatchWorld* worlds, int count, int cycles, cudaStream_t s) {
  if (count <= 0 || cycles <= 0) return cudaSuccess;
  const BatchShape sh{kClusterCtas, kClusterMaxThreads};
  // the items and the queue counter, freed in stream order after the launch
  const size_t bytes = sizeof(BatchItem) * (size_t)count + 256;
  void* d = nullptr;
  cudaError_t e = cudaMallocAsync(&d, bytes, s);
  if (e != cudaSuccess) return e;
  void* d_items = static_cast<char*>(d) + 256;
  unsigned* d_queue = static_cast<unsigned*>(d);
  const int clusters = batch_clusters(sh, count);
  e = clusters < 1 ? cudaErrorCooperativeLaunchTooLarge : upload_batch_items(worlds, count, sh, d_items, s);
  if (e == cudaSuccess) e = launch_batch_items(d_items, d_queue, count, cycles, sh, clusters, s);
  const cudaError_t es = cudaStreamSynchronize(s);
  cudaFreeAsync(d, s);
  return e != cudaSuccess ? e : es;
}

void launch_sum_fixed(const int32_t* hq, long n, long long* out, cudaStream_t s) {
  k_sum_fixed<<<sweep_grid(n), 256, 0, s>>>(hq, n, out);
}

}  // namespace swe
