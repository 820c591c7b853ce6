// Exact-semantics kernels: the reference's sequential algorithm on float
// maps, step for step.
//
//   k_ordered_particles  World::erode's particle loop (world.hpp:47-67), one
//                        thread, particles in order, rand() from the replica
//                        of the C library generator or from a caller tape.
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

// World::cascade (world.hpp:79-153): in-bounds neighbours, stable descending
// insertion sort of their heights (libstdc++ std::sort on <= 16 elements),
// then excess-over-slope transfers against the live centre height.
__device__ int cascade_exact(float* H, const Consts& c, int x, int z) {
  int sx[8], sz[8];
  float sh[8], sd[8];
  int num = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int dx = kNbDx[k], dz = kNbDz[k];
    const int qx = x + dx, qz = z + dz;
    if (oob(c, qx, qz)) continue;
    sx[num] = qx; sz[num] = qz;
    sh[num] = H[(long)qx * c.nz + qz];
    const float fx = (float)dx, fz = (float)dz;
    sd[num] = sqrtf(fx * fx + fz * fz);
    num++;
  }
  for (int i = 1; i < num; i++) {
    const int vx = sx[i], vz = sz[i];
    const float vh = sh[i], vd = sd[i];
    if (vh > sh[0]) {
      for (int j = i; j > 0; j--) { sx[j] = sx[j - 1]; sz[j] = sz[j - 1]; sh[j] = sh[j - 1]; sd[j] = sd[j - 1]; }
      sx[0] = vx; sz[0] = vz; sh[0] = vh; sd[0] = vd;
    } else {
      int j = i;
      while (vh > sh[j - 1]) { sx[j] = sx[j - 1]; sz[j] = sz[j - 1]; sh[j] = sh[j - 1]; sd[j] = sd[j - 1]; j--; }
      sx[j] = vx; sz[j] = vz; sh[j] = vh; sd[j] = vd;
    }
  }
  const long ci = (long)x * c.nz + z;
  int transfers = 0;
  for (int i = 0; i < num; i++) {
    const float diff = H[ci] - sh[i];
    if (diff == 0.0f) continue;
    const float excess = fabsf(diff) - sd[i] * c.maxdiff;
    if (excess <= 0.0f) continue;
    const float transfer = c.settling * excess / 2.0f;
    const long qi = (long)sx[i] * c.nz + sz[i];
    if (diff > 0.0f) {
      H[ci] -= transfer;
      H[qi] += transfer;
    } else {
      H[ci] += transfer;
      H[qi] -= transfer;
    }
    transfers++;
  }
  return transfers;
}

// Wind::fly (wind.hpp:28-117). With Frozen the map is only read.
template <bool Frozen, class Rand>
__device__ bool fly_exact(float* H, const Fields* F, const Consts& c, FlyState& P, Rand& rnd, int& transfers) {
  const int ix = (int)roundf(P.pos.x);
  const int iz = (int)roundf(P.pos.z);
  if (oob(c, ix, iz)) return false;
  const V3 n = surface_normal(ix, iz, c.nx, c.nz, c.mapscale,
                              [&](int a, int b) { return H[(long)a * c.nz + b]; });
  const long ci = (long)ix * c.nz + iz;
  if (P.age == 0 || P.pos.y < H[ci]) P.pos.y = H[ci];
  if (P.age++ > c.max_age) return false;

  float hfac = exp_libm(-(P.pos.y - H[ci]) / c.boundarylayer, c);
  if (hfac < 0.0f) hfac = 0.0f;

  float shadow = dot(normalize(P.pspeed), n);
  if (shadow < 0.0f) shadow = 0.0f;
  shadow = 1.0f - shadow;
  P.speed = add(P.speed, smul(0.05f, sub(smul(0.1f + 0.9f * shadow, P.pspeed), P.speed)));

  if (P.pos.y > H[ci]) P.speed.y -= c.gravity * P.sediment;

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
  const float drag = (float)(1.0 - 0.3 * (double)P.sediment);
  P.speed = v3(P.speed.x * drag, P.speed.y * drag, P.speed.z * drag);

  P.pos = add(P.pos, P.speed);

  if (!Frozen) {
    F->f[6][ci] += P.speed.x;
    F->f[7][ci] += P.speed.y;
    F->f[8][ci] += P.speed.z;
    F->f[5][ci] += P.sediment;
  }

  float force = -dot(normalize(P.speed), n) * length(P.speed);
  if (force < 0.0f) force = 0.0f;
  const float lift = (1.0f - collision) * length(P.speed);
  const float capacity = force * hfac + 0.02f * lift * hfac;

  const float diff = capacity - P.sediment;
  if (!Frozen) H[ci] -= c.suspension * diff;
  P.sediment += c.suspension * diff;

  if (!Frozen) transfers += cascade_exact(H, c, ix, iz);
  return true;
}

__device__ __forceinline__ FlyState spawn_state(const Consts& c, float x, float z) {
  FlyState P;
  P.age = 0;
  P.sediment = 0.0f;
  P.pos = v3(x, 0.0f, z);
  P.speed = v3(0.0f, 0.0f, 0.0f);
  P.pspeed = v3(c.px, c.py, c.pz);
  return P;
}

__device__ __forceinline__ void record(const FlyState& P, bool alive, float* rec) {
  rec[0] = alive ? 1.0f : 0.0f;
  rec[1] = (float)P.age;
  rec[2] = P.pos.x; rec[3] = P.pos.y; rec[4] = P.pos.z;
  rec[5] = P.speed.x; rec[6] = P.speed.y; rec[7] = P.speed.z;
  rec[8] = P.sediment;
}

__global__ void k_reset_tracks(Fields F, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    F.f[5][i] = 0.0f; F.f[6][i] = 0.0f; F.f[7][i] = 0.0f; F.f[8][i] = 0.0f;
  }
}

// cell.field = (1-lrate)*cell.field + lrate*cell.field_track (world.hpp:70-76).
__global__ void k_ema_float(Fields F, float lrate, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 1; k <= 4; k++) F.f[k][i] = (1.0f - lrate) * F.f[k][i] + lrate * F.f[k + 4][i];
  }
}

// World::erode's particle loop (world.hpp:47-67), one thread.
__global__ void k_ordered_particles(Fields F, Consts c, GlibcRandState* rng, const int32_t* tape,
                                    long long tape_len, Counters* cnt, int particles) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  OrderedRand rnd;
  rnd.g = *rng;
  rnd.tape = tape;
  rnd.tape_len = tape_len;
  rnd.pos = cnt->tape_pos;
  rnd.status = &cnt->status;
  float* H = F.f[0];
  unsigned long long steps = 0, transfers = 0;
  for (int i = 0; i < particles; i++) {
    // ivec2(rand()%res.x, rand()%res.y), then vec2(rand()%1000, rand()%1000)
    // (world.hpp:52-54): each pair's first draw is the z component.
    const int z = rnd.next() % c.nz;
    const int x = rnd.next() % c.nx;
    const int fz = rnd.next() % 1000;
    const int fx = rnd.next() % 1000;
    FlyState P = spawn_state(c, (float)x + (float)fx / 1000.0f, (float)z + (float)fz / 1000.0f);
    int tr = 0;
    while (fly_exact<false>(H, &F, c, P, rnd, tr)) steps++;
    transfers += tr;
  }
  *rng = rnd.g;
  cnt->tape_pos = rnd.pos;
  cnt->particle_steps += steps;
  cnt->particles += particles;
  cnt->transfers += transfers;
}

__global__ void k_trace(const float* H, Consts c, const float* spawn_xz, int n, int steps, const int32_t* tape,
                        float* out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  FlyState P = spawn_state(c, spawn_xz[2 * p], spawn_xz[2 * p + 1]);
  bool alive = true;
  int tr = 0;
  for (int s = 0; s < steps; s++) {
    if (alive) {
      SlotRand rnd{tape + ((long)p * steps + s) * 3, 0};
      alive = fly_exact<true>(const_cast<float*>(H), nullptr, c, P, rnd, tr);
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
  bool alive = true;
  int ok = 0, tr = 0;
  for (int s = 0; s < steps; s++) {
    if (alive) {
      if (tape) {
        SlotRand sr{tape + (long)s * 3, 0};
        alive = fly_exact<false>(F.f[0], &F, c, P, sr, tr);
      } else {
        alive = fly_exact<false>(F.f[0], &F, c, P, rnd, tr);
      }
      if (alive) ok++;
    }
    if (out) record(P, alive, out + (long)s * 9);
  }
  *rng = rnd.g;
  *ok_steps = ok;
}

__global__ void k_cascade_at(float* H, Consts c, int x, int z) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cascade_exact(H, c, x, z);
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
