// TEST INFRASTRUCTURE: compiles the reference's OWN hot-path headers into a
// CPU oracle shared library (oracle/_ref/libswe_ref_<N>.so). Only tests,
// the smoke check and the bench's reference/cpu_baseline legs may load it.
//
// What is compiled from the reference, unmodified:
//   source/wind.hpp     (Wind, Wind::fly            wind.hpp:4-117)
//   source/world.hpp    (World::erode, ::cascade    world.hpp:9-153)
//   source/include/math.h, FastNoiseLite.h, libmorton (transitively)
// and one generated copy of source/cellpool.h whose only change is
// `tilesize = 512` -> `tilesize = SWE_REF_N` (cellpool.h:186), written by
// oracle/Makefile into oracle/_ref/gen/. It is included first, so its include
// guard turns world.hpp's own `#include "cellpool.h"` into a no-op.
//
// glm (absent here) is replaced by oracle/glm_shim.hpp and the GL vertex pool
// by oracle/vertexpool_stub.hpp. libc rand() is routed through a hook so the
// harness can count / record the sequence, or feed a tape for frozen-map
// trajectories.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <iostream>
#include <vector>

#include "glm_shim.hpp"
using namespace glm;
using namespace std;
#include "vertexpool_stub.hpp"

extern "C" int swe_ref_rand_hook(void);
#define rand() swe_ref_rand_hook()

#define SWE_STR2(x) #x
#define SWE_STR(x) SWE_STR2(x)
#include SWE_STR(SWE_REF_SRC/include/FastNoiseLite.h)
#include SWE_STR(SWE_REF_SRC/include/math.h)
#include SWE_STR(SWE_REF_GEN/cellpool.h)
#include SWE_STR(SWE_REF_SRC/world.hpp)

#undef rand

// ---------------------------------------------------------------- rand hook
static int g_tape_mode = 0;           // 0: libc rand(), 1: read g_tape
static const int* g_tape = nullptr;
static long g_tape_len = 0, g_tape_pos = 0;
static int g_tape_overrun = 0;
static long g_rand_calls = 0;
static std::vector<int>* g_record = nullptr;

extern "C" int swe_ref_rand_hook(void) {
  g_rand_calls++;
  if (g_tape_mode) {
    if (g_tape_pos >= g_tape_len) { g_tape_overrun = 1; return 0; }
    return g_tape[g_tape_pos++];
  }
  int r = rand();
  if (g_record) g_record->push_back(r);
  return r;
}

// ---------------------------------------------------------------- map setup
static mappool::pool<quad::cell> g_pool;
static bool g_ready = false;

static quad::cell* cells() { return World::map.nodes[0].s.root.start; }

static void ensure_init() {
  if (g_ready) return;
  g_pool.reserve(quad::area);
  // Node construction as in map::init (cellpool.h:348-352), without GL.
  World::map.nodes[0].pos = ivec2(0);
  World::map.nodes[0].vertex = nullptr;
  World::map.nodes[0].s.root = g_pool.get(quad::tilearea / quad::lodarea);
  World::map.nodes[0].s.res = quad::tileres / quad::lodsize;
  // new cell[] leaves fields uninitialised (cellpool.h:141); zero them all.
  std::memset(cells(), 0, sizeof(quad::cell) * quad::area);
  g_ready = true;
}

static float* field_ptr(quad::cell& c, int f) {
  switch (f) {
    case 0: return &c.height;
    case 1: return &c.massflow;
    case 2: return &c.momentumx;
    case 3: return &c.momentumy;
    case 4: return &c.momentumz;
    case 5: return &c.massflow_track;
    case 6: return &c.momentumx_track;
    case 7: return &c.momentumy_track;
    default: return &c.momentumz_track;
  }
}

extern "C" {

int ref_size(void) { return quad::size; }

// quad::map::init (cellpool.h:339-430) itself, on a fresh cell pool: the
// node set-up, indexnode, then the reference's own terrain (the Gaussian bump
// normalised to [0, 0.5]); the other fields are zeroed afterwards as in
// ensure_init (new cell[] leaves them uninitialised, cellpool.h:141). Its
// progress lines go to stdout.
void ref_map_init(int seed) {
  static Vertexpool<Vertex> vp;
  static mappool::pool<quad::cell> pool;
  pool.reserve(quad::area);
  World::map.init(vp, pool, seed);
  quad::cell* c = World::map.nodes[0].s.root.start;
  for (int i = 0; i < quad::area; i++) {
    const float h = c[i].height;
    std::memset(&c[i], 0, sizeof(quad::cell));
    c[i].height = h;
  }
  g_ready = true;
}

// updatenode (cellpool.h:302-333) over the current map: 12 floats per cell
// (P, normal, T - P, B - P) into out, at index math::flatten(pos).
void ref_updatenode(float* out) {
  ensure_init();
  static Vertexpool<Vertex> vp;
  vp.capture = out;
  updatenode(vp, World::map.nodes[0]);
  vp.capture = nullptr;
}

void ref_set_field(int f, const float* src) {
  ensure_init();
  quad::cell* c = cells();
  for (int i = 0; i < quad::area; i++) *field_ptr(c[i], f) = src[i];
}

void ref_get_field(int f, float* dst) {
  ensure_init();
  quad::cell* c = cells();
  for (int i = 0; i < quad::area; i++) dst[i] = *field_ptr(c[i], f);
}

void ref_srand(unsigned seed) { srand(seed); }
long ref_rand_calls(void) { return g_rand_calls; }

// Records the next n libc rand() values (after srand) into out.
void ref_rand_sequence(int n, int* out) {
  for (int i = 0; i < n; i++) out[i] = rand();
}

// World::erode(P) exactly as the app calls it (SimpleWindErosion.cpp:217).
void ref_erode(int particles) {
  ensure_init();
  World::erode(particles);
}

// World::erode restated (world.hpp:36-77) with the prevailing wind set per
// particle after construction (the member is public, wind.hpp:13). With
// pspeed = (1,0,0) this is bitwise identical to ref_erode.
void ref_erode_pspeed(int particles, float px, float py, float pz) {
  ensure_init();
  for (auto& node : World::map.nodes)
    for (auto [cell, pos] : node.s) {
      cell.massflow_track = 0;
      cell.momentumx_track = 0;
      cell.momentumy_track = 0;
      cell.momentumz_track = 0;
    }
  for (auto& node : World::map.nodes)
    for (int i = 0; i < particles; i++) {
      glm::vec2 newpos = node.pos + ivec2(rand() % quad::tileres.x, rand() % quad::tileres.y);
      newpos += vec2(rand() % 1000, rand() % 1000) / 1000.0f;
      Wind wind(newpos);
      wind.pspeed = vec3(px, py, pz);
      while (wind.fly());
    }
  const float lrate = World::lrate;
  for (auto& node : World::map.nodes)
    for (auto [cell, pos] : node.s) {
      cell.massflow = (1.0f - lrate) * cell.massflow + lrate * cell.massflow_track;
      cell.momentumx = (1.0f - lrate) * cell.momentumx + lrate * cell.momentumx_track;
      cell.momentumy = (1.0f - lrate) * cell.momentumy + lrate * cell.momentumy_track;
      cell.momentumz = (1.0f - lrate) * cell.momentumz + lrate * cell.momentumz_track;
    }
}

// quad::_normal through map::normal (cellpool.h:200-223, 478-480).
void ref_normal(int x, int z, float* out3) {
  ensure_init();
  vec3 n = World::map.normal(ivec2(x, z));
  out3[0] = n.x; out3[1] = n.y; out3[2] = n.z;
}

// World::cascade at one cell (world.hpp:79-153); mutates heights.
void ref_cascade(int x, int z) {
  ensure_init();
  World::cascade(vec2(x, z));
}

// Record layout per step (9 floats): alive, age, pos.xyz, speed.xyz, sediment.
static void record(const Wind& w, bool alive, float* rec) {
  rec[0] = alive ? 1.0f : 0.0f;
  rec[1] = (float)w.age;
  rec[2] = w.pos.x; rec[3] = w.pos.y; rec[4] = w.pos.z;
  rec[5] = w.speed.x; rec[6] = w.speed.y; rec[7] = w.speed.z;
  rec[8] = w.sediment;
}

// Frozen-map trajectories: each particle is flown with Wind::fly, and after
// every step the 3x3 cells that fly may have written (the pre-move cell's
// tracks and height, and its cascade neighbours) are restored, so the map
// never changes. Turbulence draws come from `tape` (3 ints per step slot,
// in call order; particle p, step s uses tape[(p*steps+s)*3 ...]).
// Returns 0, or -1 if the tape ran short.
int ref_trace(int n, const float* spawn_xz, const float* pspeed, int steps,
              const int* tape, float* out) {
  ensure_init();
  quad::cell saved[9];
  g_tape_overrun = 0;
  for (int p = 0; p < n; p++) {
    Wind w(vec2(spawn_xz[2 * p], spawn_xz[2 * p + 1]));
    w.pspeed = vec3(pspeed[0], pspeed[1], pspeed[2]);
    bool alive = true;
    for (int s = 0; s < steps; s++) {
      float* rec = out + ((long)p * steps + s) * 9;
      if (!alive) { record(w, false, rec); continue; }
      const ivec2 ip = round(vec2(w.pos.x, w.pos.z));
      for (int k = 0; k < 9; k++) {
        ivec2 q = ip + ivec2(k / 3 - 1, k % 3 - 1);
        if (!World::map.oob(q)) saved[k] = *World::map.getCell(q);
      }
      g_tape = tape + ((long)p * steps + s) * 3;
      g_tape_len = 3; g_tape_pos = 0; g_tape_mode = 1;
      alive = w.fly();
      g_tape_mode = 0;
      for (int k = 0; k < 9; k++) {
        ivec2 q = ip + ivec2(k / 3 - 1, k % 3 - 1);
        if (!World::map.oob(q)) *World::map.getCell(q) = saved[k];
      }
      record(w, alive, rec);
    }
  }
  return g_tape_overrun ? -1 : 0;
}

// One particle flown on the live map (writes happen) for at most `steps`
// steps, rand() from libc (tape == NULL) or from a tape of 3 ints per step.
// Returns the number of successful fly() calls.
int ref_fly_live(float x, float z, const float* pspeed, int steps, const int* tape, float* out) {
  ensure_init();
  Wind w(vec2(x, z));
  w.pspeed = vec3(pspeed[0], pspeed[1], pspeed[2]);
  bool alive = true;
  int ok = 0;
  for (int s = 0; s < steps; s++) {
    if (alive) {
      if (tape) { g_tape = tape + (long)s * 3; g_tape_len = 3; g_tape_pos = 0; g_tape_mode = 1; }
      alive = w.fly();
      g_tape_mode = 0;
      if (alive) ok++;
    }
    if (out) record(w, alive, out + (long)s * 9);
  }
  return ok;
}

// Which constructor argument receives the k-th rand() call, for the three
// call shapes on the path (world.hpp:52, :54 and wind.hpp:83), as compiled
// by this compiler. out[0..1]: ivec2, out[2..3]: vec2, out[4..6]: vec3.
void ref_probe_order(int* out) {
  static const int t[3] = {0, 1, 2};
  g_tape = t; g_tape_len = 3; g_tape_pos = 0; g_tape_mode = 1;
  ivec2 a = ivec2(swe_ref_rand_hook() % 7, swe_ref_rand_hook() % 7);
  g_tape_pos = 0;
  vec2 b = vec2(swe_ref_rand_hook() % 1000, swe_ref_rand_hook() % 1000);
  g_tape_pos = 0;
  vec3 c = vec3(swe_ref_rand_hook() % 1001, swe_ref_rand_hook() % 1001, swe_ref_rand_hook() % 1001);
  g_tape_mode = 0;
  out[0] = a.x; out[1] = a.y; out[2] = (int)b.x; out[3] = (int)b.y;
  out[4] = (int)c.x; out[5] = (int)c.y; out[6] = (int)c.z;
}

}  // extern "C"
