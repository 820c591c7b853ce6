// Exact-semantics kernels: the reference's sequential algorithm on float
// maps, step for step.
//
//   k_ordered_particles  World::erode's particle loop (world.hpp:47-67), one
//                        thread, particles in order, rand() from the replica
//                        of the C library generator or from a caller tape.
//   k_ordered_batch      the same loop for an ensemble of worlds, one thread
//                        per world (k_sweep_batch: their two sweeps).
//   k_trace              Wind::fly on a frozen map (wind.hpp:28-117), one
//                        thread per particle, turbulence from a tape.
//   k_fly_live           one particle on the live map (unit checks).
//   k_cascade_at         World::cascade at one cell (world.hpp:79-153).
//   k_normals            quad::_normal for every cell (cellpool.h:200-223).
//   k_reset_tracks,
//   k_ema_float          the two O(cells) sweeps of World::erode
//                        (world.hpp:38-44, 70-76).
//
// Float operations follow the reference's order one by one (this file is
// compiled with -fmad=false), and exp is the C library's expf reproduced bit
// for bit (exp_libm), so these kernels compute what the reference binary
// computes.
#include "swe_device.cuh"
#include "swe_kernels.h"

namespace swe {
namespace {

struct FlyState {
  int age;
  float sediment;
  V3 pos, speed, pspeed;
  V3 pdir;  // normalize(pspeed), which no step changes
};

// rand() replica of the C library (TYPE_3 additive feedback generator).
__device__ __forceinline__ int glibc_next(GlibcRandState& g) {
  int h = g.head;
  int a = h + 3;  if (a >= 34) a -= 34;   // element i-31
  int b = h + 31; if (b >= 34) b -= 34;   // element i-3
  const uint32_t v = g.r[a] + g.r[b];
  g.r[h] = v;
  g.head = (h + 1 == 34) ? 0 : h + 1;
  return (int)(v >> 1);
}

// Random source of the ordered kernels: a tape, else the replica.
struct OrderedRand {
  GlibcRandState g;
  const int32_t* tape;
  long long tape_len;
  long long pos;
  unsigned int* status;
  __device__ int next() {
    if (tape) {
      if (pos < tape_len) return tape[pos++];
      atomicOr(status, 0x4u);  // SWE_STATUS_TAPE
      return 0;
    }
    return glibc_next(g);
  }
};

// Three raw draws per step from a fixed slot.
struct SlotRand {
  const int32_t* t;
  int k;
  __device__ int next() { return t[k++]; }
};

__device__ __forceinline__ bool oob(const Consts& c, int x, int z) {
  return x < 0 || z < 0 || x >= c.nx || z >= c.nz;
}

// Slot k of World::cascade's neighbour list (world.hpp:83-92): offsets
// (-1,-1) (-1,0) (-1,1) (0,-1) (0,1) (1,-1) (1,0) (1,1).
__device__ __forceinline__ int nb_dx(int k) { return k < 3 ? -1 : (k < 5 ? 0 : 1); }
__device__ __forceinline__ int nb_dz(int k) { return k == 3 ? -1 : (k == 4 ? 1 : (k < 3 ? k - 1 : k - 6)); }
// Index of slot k in a 3x3 neighbourhood stored row by row (centre 4).
__device__ __forceinline__ constexpr int nb_cell(int k) { return k < 4 ? k : k + 1; }

// The live map seen from one cell: the 3x3 heights around it and the cell's
// four tracks, held in registers. One thread is the only writer of its
// world while it runs World::erode's particle loop, so the values it stored
// are the values it would load back: the neighbourhood is loaded when the
// particle enters another cell and kept while it stays; every change is
// stored at once.
struct LiveMap {
  float* H;
  float* T[4];  // massflow, momentum x, y, z tracks
  int nx, nz;
  int cx = -1, cz = -1;  // the cell held (cx = -1: none)
  float h[9];            // heights of (cx-1+a, cz-1+b) at 3a+b, 0 out of bounds
  float t[4];            // the cell's tracks

  __device__ LiveMap(float* height, float* const* tracks, int nx_, int nz_) : H(height), nx(nx_), nz(nz_) {
#pragma unroll
    for (int k = 0; k < 4; k++) T[k] = tracks ? tracks[k] : nullptr;
  }
  __device__ void load_heights(int ix, int iz) {
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const int x = ix + a - 1, z = iz + b - 1;
        h[3 * a + b] = (x >= 0 && z >= 0 && x < nx && z < nz) ? H[(long)x * nz + z] : 0.0f;
      }
    cx = ix;
    cz = iz;
  }
  __device__ void enter(int ix, int iz) {
    if (ix == cx && iz == cz) return;
    load_heights(ix, iz);
    const long ci = (long)ix * nz + iz;
#pragma unroll
    for (int k = 0; k < 4; k++) t[k] = T[k][ci];
  }
  __device__ float at(int dx, int dz) const { return h[3 * (dx + 1) + (dz + 1)]; }
  // cell.massflow_track += sediment, cell.momentum*_track += speed
  // (wind.hpp:85-88, in the reference's order)
  __device__ void add_tracks(V3 speed, float sediment) {
    const long ci = (long)cx * nz + cz;
    t[1] += speed.x; T[1][ci] = t[1];
    t[2] += speed.y; T[2][ci] = t[2];
    t[3] += speed.z; T[3][ci] = t[3];
    t[0] += sediment; T[0][ci] = t[0];
  }
  __device__ void set_centre(float v) {
    h[4] = v;
    H[(long)cx * nz + cz] = v;
  }

  // World::cascade (world.hpp:79-153) at the cell held: the in-bounds
  // neighbours in slot order, sorted by descending height as libstdc++'s
  // insertion sort does, then the excess-over-slope transfers against the
  // live centre height (the neighbours, each listed once, are unchanged
  // until their turn). All indexes are unrolled, so the lists stay in
  // registers.
  __device__ int cascade(const Consts& c) {
    if (cx > 0 && cz > 0 && cx < nx - 1 && cz < nz - 1) {
      bool numbers = true;
#pragma unroll
      for (int k = 0; k < 8; k++) numbers = numbers && h[nb_cell(k)] == h[nb_cell(k)];
      if (numbers) return cascade_interior(c);
    }
    return cascade_any(c);
  }

  // Eight neighbours, none NaN: the insertion sort is then the stable sort
  // by descending height (a value above the front is above the whole sorted
  // prefix), here by an optimal 19-comparator sorting network for eight
  // inputs (Knuth, TAOCP vol. 3, 5.3.4) whose comparators order by height,
  // then by slot, a total order whose sorted sequence is the stable one.
  // The transfers run branch-free along the sorted list.
  __device__ int cascade_interior(const Consts& c) {
    // A cascade in which no neighbour moves against the current centre
    // leaves the centre, hence every neighbour, unchanged, in any order:
    // decide that first, without sorting.
    {
      const float md_side = sqrtf(1.0f) * c.maxdiff;
      const float md_diag = sqrtf(2.0f) * c.maxdiff;
      bool any = false;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const float diff = h[4] - h[nb_cell(k)];
        any |= diff != 0.0f && !(fabsf(diff) - (((0xA5 >> k) & 1) ? md_diag : md_side) <= 0.0f);
      }
      if (!any) return 0;
    }
    float ph[8];
    int pk[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      ph[k] = h[nb_cell(k)];
      pk[k] = k;
    }
    constexpr int kNet[19][2] = {{0, 2}, {1, 3}, {4, 6}, {5, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 1}, {2, 3},
                                 {4, 5}, {6, 7}, {2, 4}, {3, 5}, {1, 4}, {3, 6}, {1, 2}, {3, 4}, {5, 6}};
#pragma unroll
    for (int n = 0; n < 19; n++) {
      const int a = kNet[n][0], b = kNet[n][1];
      const bool sw = ph[b] > ph[a] || (ph[b] == ph[a] && pk[b] < pk[a]);
      const float th = sw ? ph[b] : ph[a];
      const int tk = sw ? pk[b] : pk[a];
      ph[b] = sw ? ph[a] : ph[b];
      pk[b] = sw ? pk[a] : pk[b];
      ph[a] = th;
      pk[a] = tk;
    }
    // d * maxdiff with d = sqrt(dx^2 + dz^2): 1 beside, sqrt(2) diagonal
    // (slots 0, 2, 5, 7)
    const float md_side = sqrtf(1.0f) * c.maxdiff;
    const float md_diag = sqrtf(2.0f) * c.maxdiff;
    float md[8];
#pragma unroll
    for (int q = 0; q < 8; q++) md[q] = ((0xA5 >> pk[q]) & 1) ? md_diag : md_side;
    float hc = h[4];
    float nv[8];
    unsigned moved = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      // skipped when diff == 0 or excess <= 0, as the reference's loop does
      const float diff = hc - ph[q];
      const float excess = fabsf(diff) - md[q];
      const bool go = diff != 0.0f && !(excess <= 0.0f);
      const float transfer = c.settling * excess / 2.0f;
      const bool down = diff > 0.0f;
      const float hn = down ? hc - transfer : hc + transfer;
      const float nn = down ? ph[q] + transfer : ph[q] - transfer;
      nv[q] = go ? nn : ph[q];
      hc = go ? hn : hc;
      moved |= (go ? 1u : 0u) << q;
    }
    if (!moved) return 0;
#pragma unroll
    for (int q = 0; q < 8; q++)
      if ((moved >> q) & 1) H[(long)(cx + nb_dx(pk[q])) * nz + (cz + nb_dz(pk[q]))] = nv[q];
    float hs[8];
#pragma unroll
    for (int q = 0; q < 8; q++) hs[pk[q]] = nv[q];
#pragma unroll
    for (int k = 0; k < 8; k++) h[nb_cell(k)] = hs[k];
    set_centre(hc);
    return __popc(moved);
  }

  // Any cell and any values: the in-bounds neighbours compacted in slot
  // order and libstdc++'s insertion sort step by step (a value above the
  // front moves to the front, any other one moves left while it is above
  // its left neighbour).
  __device__ int cascade_any(const Consts& c) {
    float ah[8];
    int as[8];
    int m = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      ah[k] = 0.0f;
      as[k] = 0;
    }
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int x = cx + nb_dx(k), z = cz + nb_dz(k);
      const bool in = x >= 0 && z >= 0 && x < nx && z < nz;
#pragma unroll
      for (int q = 0; q <= k; q++)
        if (in && q == m) {
          ah[q] = h[nb_cell(k)];
          as[q] = k;
        }
      m += in ? 1 : 0;
    }
#pragma unroll
    for (int i = 1; i < 8; i++) {
      if (i < m) {
        const float vh = ah[i];
        const int vs = as[i];
        if (vh > ah[0]) {
#pragma unroll
          for (int j = i; j > 0; j--) {
            ah[j] = ah[j - 1];
            as[j] = as[j - 1];
          }
          ah[0] = vh;
          as[0] = vs;
        } else {
          bool moving = true;
#pragma unroll
          for (int j = i; j > 0; j--) {
            if (moving) {
              if (vh > ah[j - 1]) {
                ah[j] = ah[j - 1];
                as[j] = as[j - 1];
              } else {
                ah[j] = vh;
                as[j] = vs;
                moving = false;
              }
            }
          }
        }
      }
    }
    float hc = h[4];
    int transfers = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      if (q < m) {
        const float diff = hc - ah[q];
        if (diff == 0.0f) continue;
        const int k = as[q];
        const int dx = nb_dx(k), dz = nb_dz(k);
        const float fx = (float)dx, fz = (float)dz;
        const float excess = fabsf(diff) - sqrtf(fx * fx + fz * fz) * c.maxdiff;
        if (excess <= 0.0f) continue;
        const float transfer = c.settling * excess / 2.0f;
        float nh;
        if (diff > 0.0f) {
          hc -= transfer;
          nh = ah[q] + transfer;
        } else {
          hc += transfer;
          nh = ah[q] - transfer;
        }
        H[(long)(cx + dx) * nz + (cz + dz)] = nh;
#pragma unroll
        for (int s = 0; s < 8; s++)
          if (s == k) h[nb_cell(s)] = nh;
        transfers++;
      }
    }
    if (transfers) set_centre(hc);
    return transfers;
  }
};

// The frozen map of the trajectory checks: read only, no tracks, no cascade.
struct FrozenMap {
  const float* H;
  int nz;
  long ci;
  __device__ void enter(int ix, int iz) { ci = (long)ix * nz + iz; }
  __device__ float at(int dx, int dz) const { return H[ci + (long)dx * nz + dz]; }
  __device__ void add_tracks(V3, float) {}
  __device__ void set_centre(float) {}
  __device__ int cascade(const Consts&) { return 0; }
};

// Wind::fly (wind.hpp:28-117), one step, on a LiveMap or a FrozenMap.
template <class Map, class Rand>
__device__ bool fly_exact(Map& m, const Consts& c, FlyState& P, Rand& rnd, int& transfers) {
  const int ix = (int)roundf(P.pos.x);
  const int iz = (int)roundf(P.pos.z);
  if (oob(c, ix, iz)) return false;
  m.enter(ix, iz);
  const V3 n = surface_normal(ix, iz, c.nx, c.nz, c.mapscale, [&](int a, int b) { return m.at(a - ix, b - iz); });
  const float hc = m.at(0, 0);
  if (P.age == 0 || P.pos.y < hc) P.pos.y = hc;
  if (P.age++ > c.max_age) return false;

  float hfac = exp_libm(-(P.pos.y - hc) / c.boundarylayer, c);
  if (hfac < 0.0f) hfac = 0.0f;

  float shadow = dot(P.pdir, n);
  if (shadow < 0.0f) shadow = 0.0f;
  shadow = 1.0f - shadow;
  P.speed = add(P.speed, smul(0.05f, sub(smul(0.1f + 0.9f * shadow, P.pspeed), P.speed)));

  if (P.pos.y > hc) P.speed.y -= c.gravity * P.sediment;

  float collision = -dot(normalize(P.speed), n);
  if (collision < 0.0f) collision = 0.0f;

  const V3 rspeed = cross(n, cross(smul(1.0f - collision, P.speed), n));
  P.speed = add(P.speed, smul(0.9f, sub(smul(shadow, mix(P.pspeed, rspeed, shadow * hfac)), P.speed)));

  // vec3(rand()%1001, rand()%1001, rand()%1001): the compiled reference
  // evaluates the arguments right to left, so the first draw is z.
  const int rz = rnd.next() % 1001;
  const int ry = rnd.next() % 1001;
  const int rx = rnd.next() % 1001;
  P.speed = add(P.speed, divs(smul(0.1f * hfac * collision, subs(v3((float)rx, (float)ry, (float)rz), 500.0f)), 500.0f));

  // speed *= (1.0f - 0.3*sediment): the factor is formed in double.
  const float drag = drag_factor(P.sediment);
  P.speed = v3(P.speed.x * drag, P.speed.y * drag, P.speed.z * drag);

  P.pos = add(P.pos, P.speed);

  m.add_tracks(P.speed, P.sediment);

  float force = -dot(normalize(P.speed), n) * length(P.speed);
  if (force < 0.0f) force = 0.0f;
  const float lift = (1.0f - collision) * length(P.speed);
  const float capacity = force * hfac + 0.02f * lift * hfac;

  const float diff = capacity - P.sediment;
  m.set_centre(hc - c.suspension * diff);
  P.sediment += c.suspension * diff;

  transfers += m.cascade(c);
  return true;
}

__device__ __forceinline__ FlyState spawn_state(const Consts& c, float x, float z) {
  FlyState P;
  P.age = 0;
  P.sediment = 0.0f;
  P.pos = v3(x, 0.0f, z);
  P.speed = v3(0.0f, 0.0f, 0.0f);
  P.pspeed = v3(c.px, c.py, c.pz);
  P.pdir = normalize(P.pspeed);
  return P;
}

__device__ __forceinline__ void record(const FlyState& P, bool alive, float* rec) {
  rec[0] = alive ? 1.0f : 0.0f;
  rec[1] = (float)P.age;
  rec[2] = P.pos.x; rec[3] = P.pos.y; rec[4] = P.pos.z;
  rec[5] = P.speed.x; rec[6] = P.speed.y; rec[7] = P.speed.z;
  rec[8] = P.sediment;
}

// The track reset of World::erode (world.hpp:38-44) at cell i.
__device__ __forceinline__ void reset_cell(const Fields& F, long i) {
  F.f[5][i] = 0.0f; F.f[6][i] = 0.0f; F.f[7][i] = 0.0f; F.f[8][i] = 0.0f;
}

// cell.field = (1-lrate)*cell.field + lrate*cell.field_track (world.hpp:70-76).
__device__ __forceinline__ void ema_cell(const Fields& F, float lrate, long i) {
#pragma unroll
  for (int k = 1; k <= 4; k++) F.f[k][i] = (1.0f - lrate) * F.f[k][i] + lrate * F.f[k + 4][i];
}

__global__ void k_reset_tracks(Fields F, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    reset_cell(F, i);
}

__global__ void k_ema_float(Fields F, float lrate, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    ema_cell(F, lrate, i);
}

// Both sweeps for a batch of worlds: world blockIdx.y, its cells strided
// over blockIdx.x.
__global__ void k_sweep_batch(const OrderedWorld* W, bool ema) {
  const OrderedWorld& w = W[blockIdx.y];
  const Fields F = w.F;
  const float lrate = w.c.lrate;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < w.n; i += (long)gridDim.x * blockDim.x) {
    if (ema) ema_cell(F, lrate, i);
    else reset_cell(F, i);
  }
}

// World::erode's particle loop (world.hpp:47-67) for one world, run by one
// thread: particle i is spawned when particle i-1 has died, so the rand()
// draws come in the reference's order (4 per spawn, then 3 per step).
__device__ void ordered_particles(const Fields& F, const Consts& c, GlibcRandState* rng, const int32_t* tape,
                                  long long tape_len, Counters* cnt, int particles) {
  OrderedRand rnd;
  rnd.g = *rng;
  rnd.tape = tape;
  rnd.tape_len = tape_len;
  rnd.pos = cnt->tape_pos;
  rnd.status = &cnt->status;
  LiveMap m(F.f[0], F.f + 5, c.nx, c.nz);
  unsigned long long steps = 0, transfers = 0;
  int tr = 0;  // the live particle's transfers
  FlyState P;
  bool alive = false;
  for (int i = 0;;) {
    if (!alive) {
      if (i == particles) break;
      i++;
      // ivec2(rand()%res.x, rand()%res.y), then vec2(rand()%1000, rand()%1000)
      // (world.hpp:52-54): each pair's first draw is the z component.
      const int z = rnd.next() % c.nz;
      const int x = rnd.next() % c.nx;
      const int fz = rnd.next() % 1000;
      const int fx = rnd.next() % 1000;
      P = spawn_state(c, (float)x + (float)fx / 1000.0f, (float)z + (float)fz / 1000.0f);
    }
    alive = fly_exact(m, c, P, rnd, tr);
    if (alive) {
      steps++;
    } else {
      transfers += tr;
      tr = 0;
    }
  }
  *rng = rnd.g;
  cnt->tape_pos = rnd.pos;
  cnt->particle_steps += steps;
  cnt->particles += particles;
  cnt->transfers += transfers;
}

__global__ void k_ordered_particles(Fields F, Consts c, GlibcRandState* rng, const int32_t* tape,
                                    long long tape_len, Counters* cnt, int particles) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ordered_particles(F, c, rng, tape, tape_len, cnt, particles);
}

// An ensemble of ORDERED worlds: one thread per world, `per_warp` worlds on
// the first lanes of each warp.
__global__ void k_ordered_batch(const OrderedWorld* W, int count, int per_warp) {
  const int lane = threadIdx.x & 31;
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  if (lane >= per_warp) return;
  const long i = warp * per_warp + lane;
  if (i >= count) return;
  const OrderedWorld& w = W[i];
  const Consts c = w.c;
  ordered_particles(w.F, c, w.rng, w.tape, w.tape_len, w.cnt, w.particles);
}

__global__ void k_trace(const float* H, Consts c, const float* spawn_xz, int n, int steps, const int32_t* tape,
                        float* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  FlyState P = spawn_state(c, spawn_xz[2 * p], spawn_xz[2 * p + 1]);
  FrozenMap m{H, c.nz, 0};
  bool alive = true;
  int tr = 0;
  for (int s = 0; s < steps; s++) {
    if (alive) {
      SlotRand rnd{tape + ((long)p * steps + s) * 3, 0};
      alive = fly_exact(m, c, P, rnd, tr);
    }
    record(P, alive, out + ((long)p * steps + s) * 9);
  }
}

__global__ void k_fly_live(Fields F, Consts c, float x, float z, int steps, const int32_t* tape,
                           GlibcRandState* rng, float* out, int* ok_steps, Counters* cnt) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  OrderedRand rnd;
  rnd.g = *rng;
  rnd.tape = nullptr;
  rnd.tape_len = 0;
  rnd.pos = 0;
  rnd.status = &cnt->status;
  FlyState P = spawn_state(c, x, z);
  LiveMap m(F.f[0], F.f + 5, c.nx, c.nz);
  bool alive = true;
  int ok = 0, tr = 0;
  for (int s = 0; s < steps; s++) {
    if (alive) {
      if (tape) {
        SlotRand sr{tape + (long)s * 3, 0};
        alive = fly_exact(m, c, P, sr, tr);
      } else {
        alive = fly_exact(m, c, P, rnd, tr);
      }
      if (alive) ok++;
    }
    if (out) record(P, alive, out + (long)s * 9);
  }
  *rng = rnd.g;
  *ok_steps = ok;
}

__global__ void k_cascade_at(float* H, Consts c, int x, int z) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  LiveMap m(H, nullptr, c.nx, c.nz);
  m.load_heights(x, z);
  m.cascade(c);
}

__global__ void k_normals(const float* H, Consts c, float* out) {
  const long n = (long)c.nx * c.nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i / c.nz), z = (int)(i % c.nz);
    const V3 v = surface_normal(x, z, c.nx, c.nz, c.mapscale, [&](int a, int b) { return H[(long)a * c.nz + b]; });
    out[3 * i + 0] = v.x; out[3 * i + 1] = v.y; out[3 * i + 2] = v.z;
  }
}

__global__ void k_expf_bits(Consts c, uint32_t first, long n, float* out) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = exp_libm(__uint_as_float(first + (uint32_t)i), c);
}

inline int sweep_grid(long n) {
  long g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace

void launch_expf_bits(const Consts& c, uint32_t first, long n, float* out, cudaStream_t s) {
  k_expf_bits<<<sweep_grid(n), 256, 0, s>>>(c, first, n, out);
}

void launch_reset_tracks(const Fields& F, long n, cudaStream_t s) {
  k_reset_tracks<<<sweep_grid(n), 256, 0, s>>>(F, n);
}
void launch_ema_float(const Fields& F, float lrate, long n, cudaStream_t s) {
  k_ema_float<<<sweep_grid(n), 256, 0, s>>>(F, lrate, n);
}
void launch_ordered_particles(const Fields& F, const Consts& c, GlibcRandState* rng, const int32_t* tape,
                              long long tape_len, Counters* cnt, int particles, cudaStream_t s) {
  k_ordered_particles<<<1, 1, 0, s>>>(F, c, rng, tape, tape_len, cnt, particles);
}

cudaError_t launch_ordered_batch(const OrderedWorld* worlds, int count, long max_cells, int cycles, int sms,
                                 cudaStream_t s) {
  if (count <= 0 || cycles <= 0) return cudaSuccess;
  if (sms < 1) sms = 1;
  // Worlds fill up to 8 warps per SM one per warp before warps take more.
  const long warps_wanted = 8L * sms;
  int per_warp = (int)((count + warps_wanted - 1) / warps_wanted);
  if (per_warp > 32) per_warp = 32;
  const long warps = (count + per_warp - 1) / per_warp;
  const int threads = 128;
  const long blocks = (warps * 32 + threads - 1) / threads;
  // The sweeps: one grid row per world (at most 65535 per launch), the
  // largest world's cells spread over the row.
  long bx = (max_cells + 255) / 256;
  const long bx_cap = (16L * sms + count - 1) / count;
  if (bx > bx_cap) bx = bx_cap;
  if (bx < 1) bx = 1;
  for (int k = 0; k < cycles; k++) {
    for (int first = 0; first < count; first += 65535) {
      const int rows = count - first < 65535 ? count - first : 65535;
      k_sweep_batch<<<dim3((unsigned)bx, (unsigned)rows), 256, 0, s>>>(worlds + first, false);
    }
    k_ordered_batch<<<(unsigned)blocks, threads, 0, s>>>(worlds, count, per_warp);
    for (int first = 0; first < count; first += 65535) {
      const int rows = count - first < 65535 ? count - first : 65535;
      k_sweep_batch<<<dim3((unsigned)bx, (unsigned)rows), 256, 0, s>>>(worlds + first, true);
    }
  }
  return cudaGetLastError();
}
void launch_trace(const float* height, const Consts& c, const float* spawn_xz, int n, int steps,
                  const int32_t* tape, float* out, cudaStream_t s) {
  k_trace<<<(n + 127) / 128, 128, 0, s>>>(height, c, spawn_xz, n, steps, tape, out);
}
void launch_fly_live(const Fields& F, const Consts& c, float x, float z, int steps, const int32_t* tape,
                     GlibcRandState* rng, float* out, int* ok_steps, Counters* cnt, cudaStream_t s) {
  k_fly_live<<<1, 1, 0, s>>>(F, c, x, z, steps, tape, rng, out, ok_steps, cnt);
}
void launch_cascade_at(float* height, const Consts& c, int x, int z, cudaStream_t s) {
  k_cascade_at<<<1, 1, 0, s>>>(height, c, x, z);
}
void launch_normals(const float* height, const Consts& c, float* out, cudaStream_t s) {
  k_normals<<<sweep_grid((long)c.nx * c.nz), 256, 0, s>>>(height, c, out);
}

}  // namespace swe
