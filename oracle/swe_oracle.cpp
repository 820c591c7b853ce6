// TEST INFRASTRUCTURE — CPU oracle for the SimpleWindErosion hot path.
//
// Part 1 restates the reference's sequential algorithm on SoA float maps,
// operation by operation (every float op in the reference's order, with the
// vector arithmetic of oracle/glm_shim.hpp):
//   so_erode      <- World::erode          source/world.hpp:36-77
//   fly<>         <- Wind::fly             source/wind.hpp:28-117
//   cascade       <- World::cascade        source/world.hpp:79-153
//   normal        <- quad::_normal         source/cellpool.h:200-223
//   oob / index   <- map::oob, math::flatten  cellpool.h:432-438, math.h:11-14
// rand() argument order: g++ (x86-64, -O2) evaluates the constructor
// arguments of ivec2(rand(),rand()), vec2(rand(),rand()) and
// vec3(rand(),rand(),rand()) right to left, so the first call of each group
// feeds the last component (probed by ref_probe_order in ref_harness.cpp and
// pinned by the bitwise oracle-vs-reference tests).
//
// Part 2 is a CPU model of the library's parallel fixed-point mode, written
// so that every float operation matches the CUDA kernel (compiled with
// -fmad=false, explicit fmaf only) bit for bit.
//
// Only tests, the smoke check and the bench's CPU legs load this file.
#include "swe_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V3 smul(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 muls(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
inline V3 subs(V3 a, float s) { return v3(a.x - s, a.y - s, a.z - s); }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float length(V3 v) { return std::sqrt(dot(v, v)); }
inline V3 normalize(V3 v) { return muls(v, 1.0f / std::sqrt(dot(v, v))); }
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline V3 mix(V3 x, V3 y, float a) { return add(muls(x, 1.0f - a), muls(y, a)); }

// ---------------------------------------------------------------- glibc rand
// The C library's rand() (TYPE_3 additive feedback generator): seed r[0],
// r[i] = 16807 r[i-1] mod (2^31-1) for i < 31, r[i] = r[i-31] for i in
// 31..33, then r[i] = r[i-31] + r[i-3] (mod 2^32); output i-344 is r[i] >> 1.
struct GlibcRand {
  uint32_t r[34];
  int pos;
  void seed(uint32_t s) {
    int32_t w = (int32_t)(s == 0 ? 1u : s);
    int32_t t[31];
    t[0] = w;
    for (int i = 1; i < 31; i++) {
      int64_t v = (16807LL * (int64_t)t[i - 1]) % 2147483647LL;
      if (v < 0) v += 2147483647LL;
      t[i] = (int32_t)v;
    }
    for (int i = 0; i < 31; i++) r[i] = (uint32_t)t[i];
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    pos = 0;  // r holds indices 0..33; next index to produce is 34
    base = 34;
    for (int i = 0; i < 310; i++) next_raw();
  }
  long base;
  uint32_t next_raw() {
    // ring of 34: index i lives at slot i % 34
    long i = base;
    uint32_t v = r[(i - 31) % 34] + r[(i - 3) % 34];
    r[i % 34] = v;
    base = i + 1;
    return v;
  }
  int next() { return (int)(next_raw() >> 1); }
};

// ---------------------------------------------------------------- exp kinds
inline float exp_libm(float x) { return std::exp(x); }        // glibc expf, as the reference
inline float exp_cr(float x) { return (float)std::exp((double)x); }  // correctly rounded

}  // namespace

// Own single-precision exp for the parallel mode: Cody-Waite reduction
// x = k ln2 + r, Taylor polynomial of degree 7 for e^r on |r| <= ln2/2 in
// Horner form with fused multiply-adds, scaling by 2^k through the exponent
// field. Results below e^-86 flush to 0. Identical on CPU and GPU because it
// uses only correctly rounded IEEE operations.
extern "C" float so_expf_poly(float x) {
  if (!(x == x)) return x;
  if (x < -86.0f) return 0.0f;
  if (x > 88.0f) return HUGE_VALF;
  float k = std::rint(x * 1.44269504f);
  float r = std::fmaf(k, -0.693145752f, x);
  r = std::fmaf(k, -1.42860677e-6f, r);
  float p = 1.98412698e-4f;
  p = std::fmaf(p, r, 1.38888889e-3f);
  p = std::fmaf(p, r, 8.33333333e-3f);
  p = std::fmaf(p, r, 4.16666667e-2f);
  p = std::fmaf(p, r, 1.66666667e-1f);
  p = std::fmaf(p, r, 0.5f);
  p = std::fmaf(p, r, 1.0f);
  p = std::fmaf(p, r, 1.0f);
  int ki = (int)k;
  uint32_t bits = (uint32_t)(ki + 127) << 23;
  float scale;
  std::memcpy(&scale, &bits, 4);
  return p * scale;
}

// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of the
// multiply-xor round function with the paper's multipliers and Weyl key
// increments.
extern "C" void so_philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                              uint32_t k1, uint32_t* out) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int round = 0; round < 10; round++) {
    uint64_t p0 = (uint64_t)M0 * c0;
    uint64_t p1 = (uint64_t)M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += W0; k1 += W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct so_world {
  int nx, nz;
  so_params p;
  std::vector<float> f[9];  // height, massflow, momx, momy, momz, 4 tracks (cellpool.h:226-240)
  int rng = SO_RNG_GLIBC;
  GlibcRand grand;
  const int32_t* tape = nullptr;
  long tape_len = 0, tape_pos = 0;
  int exp_kind = SO_EXP_LIBM;
  int64_t st_steps = 0, st_particles = 0, st_transfers = 0;
  // parallel model state
  std::vector<int32_t> hq;
  bool hq_valid = false;
  int64_t exported_q = 0;
  // which particles fly together (so_par_set_spawn_mode): 0 the library's
  // rule, freed lanes take the next ids; 1 lane k takes ids k, k + L, ...;
  // 2 a fixed schedule, particle j spawning at step floor(400 j / L)
  int spawn_mode = 0;
  float max_move = 0.0f;  // the last so_par_erode call's largest step along x or z (cells)

  int rnd() {
    switch (rng) {
      case SO_RNG_LIBC: return std::rand();
      case SO_RNG_GLIBC: return grand.next();
      default: return tape_pos < tape_len ? tape[tape_pos++] : 0;
    }
  }
  float ex(float x) const { return exp_kind == SO_EXP_CR ? exp_cr(x) : exp_libm(x); }
  bool oob(int x, int z) const { return x < 0 || z < 0 || x >= nx || z >= nz; }
  long idx(int x, int z) const { return (long)x * nz + z; }
  float h(int x, int z) const { return oob(x, z) ? 0.0f : f[0][idx(x, z)]; }
};

namespace {

// quad::_normal (cellpool.h:200-223) over a height accessor.
template <class H>
V3 normal_at(const so_world* w, int x, int z, H height) {
  V3 n = v3(0, 0, 0);
  const V3 s = v3(1.0f, w->p.mapscale, 1.0f);
  const float hp = height(x, z);
  if (!w->oob(x + 1, z + 1))
    n = add(n, cross(mulv(s, v3(0.0f, height(x, z + 1) - hp, 1.0f)),
                     mulv(s, v3(1.0f, height(x + 1, z) - hp, 0.0f))));
  if (!w->oob(x - 1, z - 1))
    n = add(n, cross(mulv(s, v3(0.0f, height(x, z - 1) - hp, -1.0f)),
                     mulv(s, v3(-1.0f, height(x - 1, z) - hp, 0.0f))));
  if (!w->oob(x + 1, z - 1))
    n = add(n, cross(mulv(s, v3(1.0f, height(x + 1, z) - hp, 0.0f)),
                     mulv(s, v3(0.0f, height(x, z - 1) - hp, -1.0f))));
  if (!w->oob(x - 1, z + 1))
    n = add(n, cross(mulv(s, v3(-1.0f, height(x - 1, z) - hp, 0.0f)),
                     mulv(s, v3(0.0f, height(x, z + 1) - hp, 1.0f))));
  if (length(n) > 0) n = normalize(n);
  return n;
}

const int NB_DX[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
const int NB_DZ[8] = {-1, 0, 1, -1, 1, -1, 0, 1};

struct Nb {
  int x, z;
  float h, d;
};

// libstdc++ std::sort on <= 16 elements is this insertion sort; with the
// strict comparator a.h > b.h it is stable.
template <class T, class Gt>
void insertion_sort_desc(T* a, int n, Gt gt) {
  for (int i = 1; i < n; i++) {
    T val = a[i];
    if (gt(val, a[0])) {
      for (int j = i; j > 0; j--) a[j] = a[j - 1];
      a[0] = val;
    } else {
      int j = i;
      while (gt(val, a[j - 1])) {
        a[j] = a[j - 1];
        j--;
      }
      a[j] = val;
    }
  }
}

// World::cascade (world.hpp:79-153).
void cascade(so_world* w, int x, int z) {
  Nb sn[8];
  int num = 0;
  for (int k = 0; k < 8; k++) {
    int nx_ = x + NB_DX[k], nz_ = z + NB_DZ[k];
    if (w->oob(nx_, nz_)) continue;
    float dx = (float)NB_DX[k], dz = (float)NB_DZ[k];
    sn[num++] = Nb{nx_, nz_, w->f[0][w->idx(nx_, nz_)], std::sqrt(dx * dx + dz * dz)};
  }
  insertion_sort_desc(sn, num, [](const Nb& a, const Nb& b) { return a.h > b.h; });
  float* H = w->f[0].data();
  const long c = w->idx(x, z);
  for (int i = 0; i < num; i++) {
    float diff = H[c] - sn[i].h;
    if (diff == 0) continue;
    float excess = std::fabs(diff) - sn[i].d * w->p.maxdiff;
    if (excess <= 0) continue;
    float transfer = w->p.settling * excess / 2.0f;
    const long q = w->idx(sn[i].x, sn[i].z);
    if (diff > 0) {
      H[c] -= transfer;
      H[q] += transfer;
    } else {
      H[c] += transfer;
      H[q] -= transfer;
    }
    w->st_transfers++;
  }
}

struct Particle {
  int age;
  float sediment;
  V3 pos, speed, pspeed;
};

// Wind::fly (wind.hpp:28-117). Frozen = no writes to the map.
template <bool Frozen>
bool fly(so_world* w, Particle& P) {
  const int ix = (int)std::round(P.pos.x);
  const int iz = (int)std::round(P.pos.z);
  if (w->oob(ix, iz)) return false;
  const V3 n = normal_at(w, ix, iz, [w](int a, int b) { return w->h(a, b); });
  const long c = w->idx(ix, iz);
  float* H = w->f[0].data();
  if (P.age == 0 || P.pos.y < H[c]) P.pos.y = H[c];
  if (P.age++ > w->p.max_age) return false;

  float hfac = w->ex(-(P.pos.y - H[c]) / w->p.boundarylayer);
  if (hfac < 0) hfac = 0;

  float shadow = dot(normalize(P.pspeed), n);
  if (shadow < 0) shadow = 0;
  shadow = 1.0f - shadow;
  P.speed = add(P.speed, smul(0.05f, sub(smul(0.1f + 0.9f * shadow, P.pspeed), P.speed)));

  if (P.pos.y > H[c]) P.speed.y -= w->p.gravity * P.sediment;

  float collision = -dot(normalize(P.speed), n);
  if (collision < 0) collision = 0;

  V3 rspeed = cross(n, cross(smul(1.0f - collision, P.speed), n));
  P.speed = add(P.speed,
                smul(0.9f, sub(smul(shadow, mix(P.pspeed, rspeed, shadow * hfac)), P.speed)));

  // vec3(rand()%1001, rand()%1001, rand()%1001): first call -> z (see header)
  const int rz = w->rnd() % 1001;
  const int ry = w->rnd() % 1001;
  const int rx = w->rnd() % 1001;
  P.speed = add(P.speed,
                divs(smul(0.1f * hfac * collision, subs(v3((float)rx, (float)ry, (float)rz), 500.0f)),
                     500.0f));

  const float drag = (float)(1.0f - 0.3 * (double)P.sediment);
  P.speed = v3(P.speed.x * drag, P.speed.y * drag, P.speed.z * drag);

  P.pos = add(P.pos, P.speed);

  if (!Frozen) {
    w->f[6][c] += P.speed.x;
    w->f[7][c] += P.speed.y;
    w->f[8][c] += P.speed.z;
    w->f[5][c] += P.sediment;
  }

  float force = -dot(normalize(P.speed), n) * length(P.speed);
  if (force < 0) force = 0;
  float lift = (1.0f - collision) * length(P.speed);
  float capacity = force * hfac + 0.02f * lift * hfac;

  float diff = capacity - P.sediment;
  if (!Frozen) H[c] -= w->p.suspension * diff;
  P.sediment += w->p.suspension * diff;

  if (!Frozen) cascade(w, ix, iz);
  return true;
}

void record(const Particle& P, bool alive, float* rec) {
  rec[0] = alive ? 1.0f : 0.0f;
  rec[1] = (float)P.age;
  rec[2] = P.pos.x; rec[3] = P.pos.y; rec[4] = P.pos.z;
  rec[5] = P.speed.x; rec[6] = P.speed.y; rec[7] = P.speed.z;
  rec[8] = P.sediment;
}

Particle spawn_at(const so_world* w, float x, float z) {
  Particle P;
  P.age = 0;
  P.sediment = 0.0f;
  P.pos = v3(x, 0.0f, z);
  P.speed = v3(0, 0, 0);
  P.pspeed = v3(w->p.pspeed[0], w->p.pspeed[1], w->p.pspeed[2]);
  return P;
}

}  // namespace

extern "C" {

void so_params_default(so_params* p) {
  p->max_age = 512;
  p->boundarylayer = 2.0f;
  p->suspension = 0.05f;
  p->gravity = 0.1f;
  p->lrate = 0.1f;
  p->maxdiff = 0.005f;
  p->settling = 1.0f;
  p->mapscale = 80.0f;
  p->pspeed[0] = 1.0f; p->pspeed[1] = 0.0f; p->pspeed[2] = 0.0f;
  p->frac_bits = 24;
  p->lanes = 0;
}

so_world* so_create(int nx, int nz, const so_params* p) {
  so_world* w = new so_world();
  w->nx = nx;
  w->nz = nz;
  if (p) w->p = *p; else so_params_default(&w->p);
  for (auto& v : w->f) v.assign((size_t)nx * nz, 0.0f);
  w->grand.seed(1);
  return w;
}

void so_destroy(so_world* w) { delete w; }
void so_set_params(so_world* w, const so_params* p) { w->p = *p; }

void so_set_field(so_world* w, int field, const float* src) {
  std::memcpy(w->f[field].data(), src, sizeof(float) * w->f[field].size());
  if (field == 0) w->hq_valid = false;
}

void so_get_field(so_world* w, int field, float* dst) {
  std::memcpy(dst, w->f[field].data(), sizeof(float) * w->f[field].size());
}

void so_set_rng(so_world* w, int rng, uint32_t seed) {
  w->rng = rng;
  if (rng == SO_RNG_GLIBC) w->grand.seed(seed);
  if (rng == SO_RNG_LIBC) std::srand(seed);
}
void so_set_exp(so_world* w, int exp_kind) { w->exp_kind = exp_kind; }
void so_set_tape(so_world* w, const int32_t* tape, long n) {
  w->tape = tape; w->tape_len = n; w->tape_pos = 0; w->rng = SO_RNG_TAPE;
}
long so_tape_pos(so_world* w) { return w->tape_pos; }

void so_stats(so_world* w, int64_t* steps, int64_t* particles, int64_t* transfers) {
  *steps = w->st_steps; *particles = w->st_particles; *transfers = w->st_transfers;
}

// World::erode(P), `cycles` times (world.hpp:36-77).
void so_erode(so_world* w, int particles, int cycles) {
  w->st_steps = w->st_particles = w->st_transfers = 0;
  const size_t n = (size_t)w->nx * w->nz;
  const float lrate = w->p.lrate;
  for (int cyc = 0; cyc < cycles; cyc++) {
    for (int k = 5; k < 9; k++) std::fill(w->f[k].begin(), w->f[k].end(), 0.0f);
    for (int i = 0; i < particles; i++) {
      // ivec2(rand()%res.x, rand()%res.y): first call -> z
      const int z = w->rnd() % w->nz;
      const int x = w->rnd() % w->nx;
      // vec2(rand()%1000, rand()%1000)/1000: first call -> z
      const int fz = w->rnd() % 1000;
      const int fx = w->rnd() % 1000;
      const float px = (float)x + (float)fx / 1000.0f;
      const float pz = (float)z + (float)fz / 1000.0f;
      Particle P = spawn_at(w, px, pz);
      w->st_particles++;
      while (fly<false>(w, P)) w->st_steps++;
    }
    float* m = w->f[1].data();
    float* mx = w->f[2].data();
    float* my = w->f[3].data();
    float* mz = w->f[4].data();
    const float* tm = w->f[5].data();
    const float* tx = w->f[6].data();
    const float* ty = w->f[7].data();
    const float* tz = w->f[8].data();
    for (size_t i = 0; i < n; i++) {
      m[i] = (1.0f - lrate) * m[i] + lrate * tm[i];
      mx[i] = (1.0f - lrate) * mx[i] + lrate * tx[i];
      my[i] = (1.0f - lrate) * my[i] + lrate * ty[i];
      mz[i] = (1.0f - lrate) * mz[i] + lrate * tz[i];
    }
  }
  w->hq_valid = false;
}

void so_normal(so_world* w, int x, int z, float* out3) {
  V3 n = normal_at(w, x, z, [w](int a, int b) { return w->h(a, b); });
  out3[0] = n.x; out3[1] = n.y; out3[2] = n.z;
}

void so_cascade(so_world* w, int x, int z) {
  cascade(w, x, z);
  w->hq_valid = false;
}

int so_trace(so_world* w, int n, const float* spawn_xz, int steps, const int32_t* tape, float* out) {
  const int saved_rng = w->rng;
  for (int p = 0; p < n; p++) {
    Particle P = spawn_at(w, spawn_xz[2 * p], spawn_xz[2 * p + 1]);
    bool alive = true;
    for (int s = 0; s < steps; s++) {
      float* rec = out + ((long)p * steps + s) * 9;
      if (alive) {
        w->tape = tape + ((long)p * steps + s) * 3;
        w->tape_len = 3; w->tape_pos = 0; w->rng = SO_RNG_TAPE;
        alive = fly<true>(w, P);
      }
      record(P, alive, rec);
    }
  }
  w->rng = saved_rng;
  return 0;
}

int so_fly_live(so_world* w, float x, float z, int steps, const int32_t* tape, float* out) {
  const int saved_rng = w->rng;
  Particle P = spawn_at(w, x, z);
  bool alive = true;
  int ok = 0;
  for (int s = 0; s < steps; s++) {
    if (alive) {
      if (tape) { w->tape = tape + (long)s * 3; w->tape_len = 3; w->tape_pos = 0; w->rng = SO_RNG_TAPE; }
      alive = fly<false>(w, P);
      w->rng = saved_rng;
      if (alive) ok++;
    }
    if (out) record(P, alive, out + (long)s * 9);
  }
  w->hq_valid = false;
  return ok;
}

void so_glibc_rand_sequence(uint32_t seed, int n, int32_t* out) {
  GlibcRand g;
  g.seed(seed);
  for (int i = 0; i < n; i++) out[i] = g.next();
}

}  // extern "C"

// ============================================================================
// Part 2: CPU model of the parallel fixed-point mode. Same definitions as the
// CUDA kernel (simplewinderosion_gb300/csrc/swe_parallel.cu). One step:
//   fly     every live particle runs Wind::fly against the heights as they
//           were at the start of the step; its exchange with its cell goes
//           into a delta map D and its cell's owed cascade into a visit map C
//           (integers).
//   apply   H += D for every cell.
//   cascade for the nine cell colours (x%3, z%3) in order, every cell with
//           C > 0 runs World::cascade up to C times on the current heights
//           (stopping early once a cascade moves nothing: repeating it could
//           not change anything). Cells of one colour touch disjoint 3x3
//           neighbourhoods, so each colour is free of conflicts and the order
//           of the whole step is fixed.
// ============================================================================
namespace {

int32_t to_fixed(float v) {
  if (v != v) return 0;
  if (v >= 2147483648.0f) return INT32_MAX;
  if (v < -2147483648.0f) return INT32_MIN;
  return (int32_t)std::lrintf(v);
}
int64_t to_fixed64(float v) {
  if (v != v) return 0;
  if (v >= 9223372036854775808.0f) return INT64_MAX;
  if (v < -9223372036854775808.0f) return INT64_MIN;
  return (int64_t)std::llrintf(v);
}
inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

struct PState {
  int id, age, sed_q;
  float px, py, pz, vx, vy, vz;
};

struct ParCtx {
  so_world* w;
  const int32_t* H;
  int32_t* D;
  int32_t* C;
  int64_t* tq[4];
  uint32_t seed_lo, seed_hi, c_lo, c_hi;
  int64_t exported, steps, transfers;
  float max_move = 0.0f;  // largest |step| of a particle along x or z
};

// One step of one particle against the step-start heights; true if alive.
// Turbulence draws are keyed by (particle, age after this step's increment).
bool par_fly(ParCtx& X, PState& P) {
  so_world* w = X.w;
  const so_params& c = w->p;
  const int nx = w->nx, nz = w->nz;
  const float scale = (float)(1u << c.frac_bits);
  const float inv = 1.0f / scale;
  const float sed = (float)P.sed_q * inv;
  const bool inrange = std::fabs(P.px) < 1073741824.0f && std::fabs(P.pz) < 1073741824.0f;
  const int ix = inrange ? (int)std::round(P.px) : -1;
  const int iz = inrange ? (int)std::round(P.pz) : -1;
  if (ix < 0 || iz < 0 || ix >= nx || iz >= nz) return false;
  const bool vx0 = ix > 0, vx2 = ix + 1 < nx, vz0 = iz > 0, vz2 = iz + 1 < nz;
  const long ci = (long)ix * nz + iz;
  const float h11 = (float)X.H[ci] * inv;
  const float h01 = vx0 ? (float)X.H[ci - nz] * inv : 0.0f;
  const float h21 = vx2 ? (float)X.H[ci + nz] * inv : 0.0f;
  const float h10 = vz0 ? (float)X.H[ci - 1] * inv : 0.0f;
  const float h12 = vz2 ? (float)X.H[ci + 1] * inv : 0.0f;
  V3 n = v3(0.0f, 0.0f, 0.0f);
  const V3 s = v3(1.0f, c.mapscale, 1.0f);
  if (vx2 && vz2) n = add(n, cross(mulv(s, v3(0.0f, h12 - h11, 1.0f)), mulv(s, v3(1.0f, h21 - h11, 0.0f))));
  if (vx0 && vz0) n = add(n, cross(mulv(s, v3(0.0f, h10 - h11, -1.0f)), mulv(s, v3(-1.0f, h01 - h11, 0.0f))));
  if (vx2 && vz0) n = add(n, cross(mulv(s, v3(1.0f, h21 - h11, 0.0f)), mulv(s, v3(0.0f, h10 - h11, -1.0f))));
  if (vx0 && vz2) n = add(n, cross(mulv(s, v3(-1.0f, h01 - h11, 0.0f)), mulv(s, v3(0.0f, h12 - h11, 1.0f))));
  if (length(n) > 0.0f) n = normalize(n);

  float py = P.py;
  if (P.age == 0 || py < h11) py = h11;
  P.py = py;
  if (P.age++ > c.max_age) return false;
  float hfac = so_expf_poly(-(py - h11) / c.boundarylayer);
  if (hfac < 0.0f) hfac = 0.0f;
  const V3 ps = v3(c.pspeed[0], c.pspeed[1], c.pspeed[2]);
  V3 sp = v3(P.vx, P.vy, P.vz);
  float shadow = dot(normalize(ps), n);
  if (shadow < 0.0f) shadow = 0.0f;
  shadow = 1.0f - shadow;
  sp = add(sp, smul(0.05f, sub(smul(0.1f + 0.9f * shadow, ps), sp)));
  if (py > h11) sp.y -= c.gravity * sed;
  float collision = -dot(normalize(sp), n);
  if (collision < 0.0f) collision = 0.0f;
  const V3 rs = cross(n, cross(smul(1.0f - collision, sp), n));
  sp = add(sp, smul(0.9f, sub(smul(shadow, mix(ps, rs, shadow * hfac)), sp)));
  uint32_t u[4];
  so_philox4x32((uint32_t)P.id, (uint32_t)P.age, X.c_lo, X.c_hi, X.seed_lo, X.seed_hi, u);
  const float rx = (float)(int)(u[0] % 1001u), ry = (float)(int)(u[1] % 1001u), rz = (float)(int)(u[2] % 1001u);
  sp = add(sp, divs(smul(0.1f * hfac * collision, subs(v3(rx, ry, rz), 500.0f)), 500.0f));
  const float drag = 1.0f - 0.3f * sed;
  sp = v3(sp.x * drag, sp.y * drag, sp.z * drag);
  const float px = P.px + sp.x, pz = P.pz + sp.z;
  X.max_move = std::fmax(X.max_move, std::fmax(std::fabs(sp.x), std::fabs(sp.z)));
  py = py + sp.y;
  float force = -dot(normalize(sp), n) * length(sp);
  if (force < 0.0f) force = 0.0f;
  const float lift = (1.0f - collision) * length(sp);
  const float capacity = force * hfac + 0.02f * lift * hfac;
  const float diff = capacity - sed;
  if (!(std::isfinite(diff) && std::isfinite(px) && std::isfinite(py) && std::isfinite(pz))) return false;
  const float two32 = 4294967296.0f;
  X.tq[0][ci] += to_fixed64(sed * two32);
  X.tq[1][ci] += to_fixed64(sp.x * two32);
  X.tq[2][ci] += to_fixed64(sp.y * two32);
  X.tq[3][ci] += to_fixed64(sp.z * two32);
  const int32_t ex_q = to_fixed(c.suspension * diff * scale);
  X.D[ci] = wsub(X.D[ci], ex_q);
  X.C[ci] += 1;
  P.sed_q = wadd(P.sed_q, ex_q);
  P.px = px; P.py = py; P.pz = pz;
  P.vx = sp.x; P.vy = sp.y; P.vz = sp.z;
  X.steps++;
  return true;
}

// World::cascade in fixed point at cell (x, z) of the map H: in-bounds
// neighbours in the reference's order, stable descending by height, each
// moving half the excess over the slope limit. Returns the number of
// transfers that moved a non-zero amount.
int cascade_q(so_world* w, int32_t* H, int x, int z, float scale, float inv) {
  const so_params& c = w->p;
  const int nx = w->nx, nz = w->nz;
  struct K { int k; int32_t key; };
  K sn[8];
  int num = 0;
  for (int k = 0; k < 8; k++) {
    const int qx = x + NB_DX[k], qz = z + NB_DZ[k];
    if (qx < 0 || qz < 0 || qx >= nx || qz >= nz) continue;
    sn[num++] = K{k, H[(long)qx * nz + qz]};
  }
  insertion_sort_desc(sn, num, [](const K& a, const K& b) { return a.key > b.key; });
  int32_t& hc = H[(long)x * nz + z];
  int t = 0;
  for (int r = 0; r < num; r++) {
    const int k = sn[r].k;
    const float dx = (float)NB_DX[k], dz = (float)NB_DZ[k];
    const float d = std::sqrt(dx * dx + dz * dz);
    const int32_t dq = wsub(hc, sn[r].key);
    if (dq == 0) continue;
    const float excess = std::fabs((float)dq * inv) - d * c.maxdiff;
    if (excess <= 0.0f) continue;
    const int32_t tq = to_fixed(c.settling * excess * 0.5f * scale);
    if (tq == 0) continue;
    const int32_t sgn = dq > 0 ? tq : -tq;
    int32_t& hn = H[(long)(x + NB_DX[k]) * nz + (z + NB_DZ[k])];
    hc = wsub(hc, sgn);
    hn = wadd(hn, sgn);
    t++;
  }
  return t;
}

// The cascade phase of one step: nine colours, each cell's owed cascades.
int64_t cascade_phase(so_world* w, int32_t* H, int32_t* C) {
  const int nx = w->nx, nz = w->nz;
  const float scale = (float)(1u << w->p.frac_bits);
  const float inv = 1.0f / scale;
  int64_t transfers = 0;
  for (int col = 0; col < 9; col++)
    for (int x = col / 3; x < nx; x += 3)
      for (int z = col % 3; z < nz; z += 3) {
        const long g = (long)x * nz + z;
        const int cnt = C[g];
        C[g] = 0;
        for (int r = 0; r < cnt; r++) {
          const int t = cascade_q(w, H, x, z, scale, inv);
          if (t == 0) break;
          transfers += t;
        }
      }
  return transfers;
}

void ensure_fixed(so_world* w) {
  if (w->hq_valid) return;
  const size_t n = (size_t)w->nx * w->nz;
  const float scale = (float)(1u << w->p.frac_bits);
  w->hq.resize(n);
  for (size_t i = 0; i < n; i++) w->hq[i] = to_fixed(w->f[0][i] * scale);
  w->hq_valid = true;
  w->exported_q = 0;
}

}  // namespace

extern "C" {

int so_par_lanes(int lanes, int nx, int nz, int particles) {
  long l;
  if (lanes > 0) l = lanes;
  else if (lanes == 0) {
    l = (long)nx * nz / 256;
    if (l < 1024) l = 1024;
  } else l = particles;
  if (l > particles) l = particles;
  return (int)(l < 1 ? 1 : l);
}

void so_par_erode(so_world* w, int particles, int cycles, uint64_t seed, uint64_t* cycle_counter) {
  ensure_fixed(w);
  const size_t n = (size_t)w->nx * w->nz;
  const float inv = 1.0f / (float)(1u << w->p.frac_bits);
  const float lrate = w->p.lrate;
  std::vector<int64_t> tq[4];
  for (auto& t : tq) t.assign(n, 0);
  std::vector<int32_t> D(n, 0), C(n, 0);
  std::vector<PState> live, next;
  w->st_steps = w->st_particles = w->st_transfers = 0;
  w->max_move = 0.0f;
  for (int cyc = 0; cyc < cycles; cyc++) {
    const uint64_t cc = *cycle_counter;
    ParCtx X;
    X.w = w;
    X.seed_lo = (uint32_t)seed; X.seed_hi = (uint32_t)(seed >> 32);
    X.c_lo = (uint32_t)cc; X.c_hi = (uint32_t)(cc >> 32);
    X.exported = X.steps = X.transfers = 0;
    for (auto& t : tq) std::fill(t.begin(), t.end(), 0);
    for (int k = 0; k < 4; k++) X.tq[k] = tq[k].data();
    X.D = D.data();
    X.C = C.data();
    live.clear();
    const int lanes = so_par_lanes(w->p.lanes, w->nx, w->nz, particles);
    const int mode = w->spawn_mode;
    int next_id = 0;
    std::vector<int> lane_of, next_lane, lane_next(lanes);
    auto spawn = [&](int i, int lane) {
      uint32_t u[4];
      so_philox4x32((uint32_t)i, 0xFFFFFFFFu, X.c_lo, X.c_hi, X.seed_lo, X.seed_hi, u);
      const int x = (int)(u[0] % (uint32_t)w->nx), z = (int)(u[1] % (uint32_t)w->nz);
      const int fxq = (int)(u[2] % 1000u), fzq = (int)(u[3] % 1000u);
      PState P;
      P.id = i; P.age = 0; P.sed_q = 0;
      P.px = (float)x + (float)fxq / 1000.0f; P.py = 0.0f; P.pz = (float)z + (float)fzq / 1000.0f;
      P.vx = P.vy = P.vz = 0.0f;
      live.push_back(P);
      lane_of.push_back(lane);
    };
    // the fixed schedule's spawns up to step s: ids j with 400 j < (s + 1) L
    constexpr long kLife = 400;
    auto spawn_scheduled = [&](long s) {
      while (next_id < particles && (long)next_id * kLife < (s + 1) * (long)lanes) {
        spawn(next_id, 0);
        next_id++;
      }
    };
    if (mode == 2) {
      spawn_scheduled(0);
    } else if (mode == 1) {
      for (int k = 0; k < lanes && k < particles; k++) {
        spawn(k, k);
        lane_next[k] = k + lanes;
      }
    } else {
      while (next_id < particles && (int)live.size() < lanes) {
        spawn(next_id, (int)live.size());
        next_id++;
      }
    }
    long step = 0;
    std::vector<int> freed;
    while (!live.empty() || (mode == 2 && next_id < particles)) {
      X.H = w->hq.data();
      next.clear();
      next_lane.clear();
      freed.clear();
      for (size_t q = 0; q < live.size(); q++) {
        PState& P = live[q];
        if (par_fly(X, P)) {
          next.push_back(P);
          next_lane.push_back(lane_of[q]);
        } else {
          X.exported += P.sed_q;
          freed.push_back(lane_of[q]);
        }
      }
      if (!next.empty()) {
        int32_t* H = w->hq.data();
        for (size_t i = 0; i < n; i++) {
          H[i] = wadd(H[i], D[i]);
          D[i] = 0;
        }
        X.transfers += cascade_phase(w, H, C.data());
      }
      live.swap(next);
      lane_of.swap(next_lane);
      step++;
      // the particles of the next step: they fly from the next step
      if (mode == 2) {
        spawn_scheduled(step);
      } else if (mode == 1) {
        for (int lane : freed)
          if (lane_next[lane] < particles) {
            spawn(lane_next[lane], lane);
            lane_next[lane] += lanes;
          }
      } else {
        for (int lane : freed)
          if (next_id < particles) {
            spawn(next_id, lane);
            next_id++;
          }
      }
    }
    for (size_t i = 0; i < n; i++) {
      for (int k = 0; k < 4; k++) {
        const float t = (float)tq[k][i] * 2.3283064365386963e-10f;
        w->f[5 + k][i] = t;
        w->f[1 + k][i] = (1.0f - lrate) * w->f[1 + k][i] + lrate * t;
      }
      w->f[0][i] = (float)w->hq[i] * inv;
    }
    w->exported_q += X.exported;
    w->max_move = std::fmax(w->max_move, X.max_move);
    w->st_steps += X.steps;
    w->st_particles += particles;
    w->st_transfers += X.transfers;
    *cycle_counter = cc + 1;
  }
}

void so_par_set_spawn_mode(so_world* w, int mode) { w->spawn_mode = mode < 0 || mode > 2 ? 0 : mode; }

float so_par_max_move(so_world* w) { return w->max_move; }

void so_par_get_heights_q(so_world* w, int32_t* dst) {
  ensure_fixed(w);
  std::memcpy(dst, w->hq.data(), sizeof(int32_t) * w->hq.size());
}

void so_par_ledger(so_world* w, int64_t* map_q, int64_t* exported_q) {
  ensure_fixed(w);
  int64_t s = 0;
  for (int32_t v : w->hq) s += v;
  *map_q = s;
  *exported_q = w->exported_q;
}

}  // extern "C"

extern "C" void so_expf_libm_bits(uint32_t first, long n, float* out) {
  for (long i = 0; i < n; i++) {
    const uint32_t u = first + (uint32_t)i;
    float x;
    std::memcpy(&x, &u, 4);
    out[i] = std::exp(x);
  }
}
