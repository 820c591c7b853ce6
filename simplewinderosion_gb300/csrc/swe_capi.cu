// C ABI of the library (include/swe.h): the world object that owns the
// device-resident cell maps and drives the kernels on its own stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "swe.h"
#include "swe_kernels.h"

using swe::Consts;
using swe::Counters;
using swe::Fields;
using swe::GlibcRandState;

// The build-time list of arguments where the C library expf is not the
// correctly rounded value (swe_libm_table.cpp, gen_libm_expf.cpp):
// uint32 count, count sorted uint32 bit patterns, count int8 directions.
extern "C" const unsigned char swe_libm_expf_blob[];
extern "C" const unsigned char swe_libm_expf_blob_end[];

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

#define SWE_CK(call)                                                                    \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      return fail(e_ == cudaErrorMemoryAllocation ? SWE_ERR_NO_MEMORY : SWE_ERR_CUDA,   \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                  \
    }                                                                                   \
  } while (0)

// Host side of the C library rand() replica (same recurrence as the device
// side in swe_exact.cu): seeds r[0] = seed, r[i] = 16807 r[i-1] mod (2^31-1)
// for i < 31, r[i] = r[i-31] for i = 31..33, then discards 310 elements of
// r[i] = r[i-31] + r[i-3].
uint32_t glibc_step(GlibcRandState& g) {
  int h = g.head;
  int a = h + 3;  if (a >= 34) a -= 34;
  int b = h + 31; if (b >= 34) b -= 34;
  const uint32_t v = g.r[a] + g.r[b];
  g.r[h] = v;
  g.head = (h + 1 == 34) ? 0 : h + 1;
  return v;
}

void glibc_seed(GlibcRandState& g, uint32_t seed) {
  const int32_t s = (int32_t)(seed == 0 ? 1u : seed);
  int32_t t[31];
  t[0] = s;
  for (int i = 1; i < 31; i++) {
    long long v = (16807LL * (long long)t[i - 1]) % 2147483647LL;
    if (v < 0) v += 2147483647LL;
    t[i] = (int32_t)v;
  }
  for (int i = 0; i < 31; i++) g.r[i] = (uint32_t)t[i];
  for (int i = 31; i < 34; i++) g.r[i] = g.r[i - 31];
  g.head = 0;  // element 34 goes to slot 0
  g.pad = 0;
  for (int i = 0; i < 310; i++) glibc_step(g);
}

bool params_ok(const swe_params& p, std::string& why) {
  if (p.max_age < 0 || p.max_age > 1000000) { why = "max_age must be in [0, 1e6]"; return false; }
  if (p.frac_bits < 8 || p.frac_bits > 28) { why = "frac_bits must be in [8, 28]"; return false; }
  if (!(p.boundarylayer != 0.0f)) { why = "boundarylayer must be non-zero"; return false; }
  return true;
}

}  // namespace

void swe::set_last_error(const std::string& msg) { g_error = msg; }

struct swe_world {
  int nx = 0, nz = 0;
  long n = 0;
  swe_params p{};
  uint64_t seed = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  Fields F{};
  float* fbase = nullptr;
  Counters* cnt = nullptr;
  GlibcRandState* grand = nullptr;
  int32_t* tape = nullptr;
  long long tape_len = 0;
  // parallel mode
  int32_t* hq = nullptr;      // heights; deltas, visit counts, owners of even and odd steps; 3 visited bitmaps
  long long* tq = nullptr;    // 4n
  unsigned long long* hw = nullptr;  // n height words of the bounded-lanes form, one padding word each side
  void* pstate = nullptr;     // 2 buffers x 9 arrays x capacity
  int pcap = 0;
  swe::ParallelBuffers pb{};
  bool hq_valid = false;
  int cycle_grid = 0;
  long long* dsum = nullptr;
  swe::GridBarrier* gbar = nullptr;
  bool own_stream = true;
  uint32_t* expf_x = nullptr;  // device copy of the expf exception list
  int8_t* expf_d = nullptr;
  int expf_n = 0;
  uint64_t wait_ns = 0;  // parallel-mode wait deadline (0: the default, 2 s)
  // An aborted parallel cycle (SWE_STATUS_TIMEOUT) leaves deltas and visit
  // counts behind in maps that every cycle expects at zero; the next
  // parallel call clears them first.
  bool scratch_dirty = false;
  swe::LaunchForm form;  // bounded-lanes launch form (default: the library's rule)

  Consts consts() const {
    Consts c;
    c.nx = nx; c.nz = nz;
    c.max_age = p.max_age;
    c.boundarylayer = p.boundarylayer; c.suspension = p.suspension; c.gravity = p.gravity;
    c.lrate = p.lrate; c.maxdiff = p.maxdiff; c.settling = p.settling; c.mapscale = p.mapscale;
    c.px = p.pspeed[0]; c.py = p.pspeed[1]; c.pz = p.pspeed[2];
    c.frac_bits = p.frac_bits;
    c.scale = (float)(1u << p.frac_bits);
    c.inv_scale = 1.0f / c.scale;
    c.expf_x = expf_x;
    c.expf_d = expf_d;
    c.expf_n = expf_n;
    c.wait_ns = wait_ns;
    return c;
  }

};

namespace {

int use_device(swe_world* w) {
  SWE_CK(cudaSetDevice(w->device));
  return SWE_OK;
}

// Parallel-mode buffers, grown to hold `particles` in flight.
int ensure_parallel(swe_world* w, int particles) {
  // heights, then exchange deltas and visit counts of even and odd steps,
  // the cell owners of both, each padded to 64 elements so every map starts
  // 256-byte aligned; then three visited bitmaps.
  const size_t stride = ((size_t)w->n + 63) & ~(size_t)63;
  const size_t bw = ((size_t)(w->n + 128) / 32 + 2 + 63) & ~(size_t)63;
  if (!w->hq) {
    SWE_CK(cudaMalloc(&w->hq, sizeof(int32_t) * (7 * stride + 3 * bw)));
    SWE_CK(cudaMemsetAsync(w->hq, 0, sizeof(int32_t) * (7 * stride + 3 * bw), w->stream));
    SWE_CK(cudaMalloc(&w->tq, sizeof(long long) * 4 * w->n));
    SWE_CK(cudaMalloc(&w->hw, sizeof(unsigned long long) * (w->n + 2)));
    SWE_CK(cudaMemsetAsync(w->tq, 0, sizeof(long long) * 4 * w->n, w->stream));
    SWE_CK(cudaMalloc(&w->dsum, sizeof(long long)));
    SWE_CK(cudaMalloc(&w->gbar, sizeof(swe::GridBarrier)));
    SWE_CK(cudaMemsetAsync(w->gbar, 0, sizeof(swe::GridBarrier), w->stream));
    w->cycle_grid = swe::cycle_grid(w->device);
    if (w->cycle_grid < 1) return fail(SWE_ERR_CUDA, "device cannot run the cooperative cycle kernel");
  }
  if (particles > w->pcap || !w->pstate) {
    const int cap = particles > 0 ? particles : 1;
    if (w->pstate) SWE_CK(cudaFree(w->pstate));
    w->pstate = nullptr;
    SWE_CK(cudaMalloc(&w->pstate, sizeof(int32_t) * 9 * 2 * (size_t)cap));
    w->pcap = cap;
  }
  swe::ParallelBuffers& B = w->pb;
  B.hq = w->hq;
  B.dq = w->hq + stride;
  B.visits = w->hq + 2 * stride;
  B.dq2 = w->hq + 3 * stride;
  B.visits2 = w->hq + 4 * stride;
  B.owner = w->hq + 5 * stride;
  B.owner2 = w->hq + 6 * stride;
  for (int k = 0; k < 3; k++) B.vbits[k] = reinterpret_cast<uint32_t*>(w->hq + 7 * stride + k * bw);
  B.vbits_words = (long)((w->n + 128) / 32 + 2);
  B.hw = w->hw + 1;
  for (int k = 0; k < 4; k++) B.tq[k] = w->tq + (size_t)k * w->n;
  int32_t* base = reinterpret_cast<int32_t*>(w->pstate);
  for (int b = 0; b < 2; b++) {
    int32_t* s = base + (size_t)b * 9 * w->pcap;
    swe::ParticleSoA& S = B.state[b];
    S.id = s;
    S.age = s + 1 * (size_t)w->pcap;
    S.px = reinterpret_cast<float*>(s + 2 * (size_t)w->pcap);
    S.py = reinterpret_cast<float*>(s + 3 * (size_t)w->pcap);
    S.pz = reinterpret_cast<float*>(s + 4 * (size_t)w->pcap);
    S.vx = reinterpret_cast<float*>(s + 5 * (size_t)w->pcap);
    S.vy = reinterpret_cast<float*>(s + 6 * (size_t)w->pcap);
    S.vz = reinterpret_cast<float*>(s + 7 * (size_t)w->pcap);
    S.sed_q = s + 8 * (size_t)w->pcap;
  }
  B.capacity = w->pcap;
  return SWE_OK;
}

int ensure_fixed(swe_world* w) {
  if (w->hq_valid) return SWE_OK;
  const Consts c = w->consts();
  swe::launch_height_to_fixed(w->F.f[0], w->pb.hq, c, w->cnt, w->stream);
  SWE_CK(cudaGetLastError());
  w->hq_valid = true;
  return SWE_OK;
}

// After an aborted cycle: zero the deltas and visit counts of even and odd
// steps (the maps after the heights), which a finished cycle leaves at zero.
int clear_after_abort(swe_world* w) {
  if (!w->scratch_dirty) return SWE_OK;
  w->scratch_dirty = false;
  const size_t stride = ((size_t)w->n + 63) & ~(size_t)63;
  SWE_CK(cudaMemsetAsync(w->pb.dq, 0, sizeof(int32_t) * 4 * stride, w->stream));
  return SWE_OK;
}

// Enqueue one parallel erode cycle: reset the grid barrier, then the
// persistent cooperative kernel (spawn, steps, EMA).
int enqueue_parallel_cycle(swe_world* w, int particles, int lanes) {
  SWE_CK(cudaMemsetAsync(w->gbar, 0, sizeof(swe::GridBarrier), w->stream));
  SWE_CK(swe::launch_par_cycle(w->pb, w->F, w->consts(), w->seed, w->cnt, w->gbar, particles, lanes,
                               w->cycle_grid, w->stream, w->form));
  return SWE_OK;
}

std::mutex g_form_mutex;
std::map<std::string, swe::LaunchForm> g_forms;  // (sides, particles, lanes) -> fastest form

}  // namespace

extern "C" {

void swe_params_default(swe_params* p) {
  if (!p) return;
  p->max_age = 512;
  p->boundarylayer = 2.0f;
  p->suspension = 0.05f;
  p->gravity = 0.1f;
  p->lrate = 0.1f;
  p->maxdiff = 0.005f;
  p->settling = 1.0f;
  p->mapscale = 80.0f;
  p->pspeed[0] = 1.0f;
  p->pspeed[1] = 0.0f;
  p->pspeed[2] = 0.0f;
  p->frac_bits = 24;
  p->lanes = 0;
}

const char* swe_last_error(void) { return g_error.c_str(); }

int swe_world_create(int nx, int nz, const swe_params* p, uint64_t seed, swe_world** out) {
  if (!out) return fail(SWE_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (nx < 1 || nz < 1) return fail(SWE_ERR_INVALID, "nx and nz must be >= 1");
  if ((long long)nx * nz >= (1LL << 31)) return fail(SWE_ERR_INVALID, "nx*nz must be < 2^31");
  swe_params prm;
  if (p) prm = *p; else swe_params_default(&prm);
  std::string why;
  if (!params_ok(prm, why)) return fail(SWE_ERR_INVALID, why);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(SWE_ERR_CUDA, "no CUDA device available");
  }
  swe_world* w = new swe_world();
  w->nx = nx; w->nz = nz; w->n = (long)nx * nz;
  w->p = prm;
  w->seed = seed;
  int rc = SWE_OK;
  auto init = [&]() -> int {
    SWE_CK(cudaGetDevice(&w->device));
    SWE_CK(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
    SWE_CK(cudaMalloc(&w->fbase, sizeof(float) * 9 * (size_t)w->n));
    for (int k = 0; k < 9; k++) w->F.f[k] = w->fbase + (size_t)k * w->n;
    SWE_CK(cudaMemsetAsync(w->fbase, 0, sizeof(float) * 9 * (size_t)w->n, w->stream));
    SWE_CK(cudaMalloc(&w->cnt, sizeof(Counters)));
    SWE_CK(cudaMemsetAsync(w->cnt, 0, sizeof(Counters), w->stream));
    {
      uint32_t cnt = 0;
      std::memcpy(&cnt, swe_libm_expf_blob, 4);
      const size_t blob = (size_t)(swe_libm_expf_blob_end - swe_libm_expf_blob);
      if (blob != 4 + 5 * (size_t)cnt) return fail(SWE_ERR_INVALID, "embedded expf table is malformed");
      w->expf_n = (int)cnt;
      SWE_CK(cudaMalloc(&w->expf_x, 4 * (size_t)cnt + 4));
      SWE_CK(cudaMalloc(&w->expf_d, (size_t)cnt + 4));
      SWE_CK(cudaMemcpyAsync(w->expf_x, swe_libm_expf_blob + 4, 4 * (size_t)cnt, cudaMemcpyHostToDevice, w->stream));
      SWE_CK(cudaMemcpyAsync(w->expf_d, swe_libm_expf_blob + 4 + 4 * (size_t)cnt, cnt, cudaMemcpyHostToDevice,
                             w->stream));
    }
    SWE_CK(cudaMalloc(&w->grand, sizeof(GlibcRandState)));
    GlibcRandState g;
    glibc_seed(g, (uint32_t)seed);
    SWE_CK(cudaMemcpyAsync(w->grand, &g, sizeof(g), cudaMemcpyHostToDevice, w->stream));
    SWE_CK(cudaStreamSynchronize(w->stream));
    return SWE_OK;
  };
  rc = init();
  if (rc != SWE_OK) {
    std::string msg = g_error;
    swe_world_destroy(w);
    g_error = msg;
    return rc;
  }
  *out = w;
  return SWE_OK;
}

void swe_world_destroy(swe_world* w) {
  if (!w) return;
  cudaSetDevice(w->device);
  if (w->stream) cudaStreamSynchronize(w->stream);
  cudaFree(w->fbase);
  cudaFree(w->cnt);
  cudaFree(w->grand);
  cudaFree(w->tape);
  cudaFree(w->hq);
  cudaFree(w->tq);
  cudaFree(w->hw);
  cudaFree(w->pstate);
  cudaFree(w->dsum);
  cudaFree(w->gbar);
  cudaFree(w->expf_x);
  cudaFree(w->expf_d);
  if (w->stream && w->own_stream) cudaStreamDestroy(w->stream);
  delete w;
}

int swe_world_set_params(swe_world* w, const swe_params* p) {
  if (!w || !p) return fail(SWE_ERR_INVALID, "NULL argument");
  std::string why;
  if (!params_ok(*p, why)) return fail(SWE_ERR_INVALID, why);
  if (p->frac_bits != w->p.frac_bits) w->hq_valid = false;
  w->p = *p;
  return SWE_OK;
}

int swe_world_get_params(swe_world* w, swe_params* p) {
  if (!w || !p) return fail(SWE_ERR_INVALID, "NULL argument");
  *p = w->p;
  return SWE_OK;
}

int swe_world_size(swe_world* w, int* nx, int* nz) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (nx) *nx = w->nx;
  if (nz) *nz = w->nz;
  return SWE_OK;
}

int swe_world_upload(swe_world* w, swe_field f, const float* host, size_t n) {
  if (!w || !host) return fail(SWE_ERR_INVALID, "NULL argument");
  if ((int)f < 0 || (int)f > 8) return fail(SWE_ERR_INVALID, "unknown field");
  if (n != (size_t)w->n) return fail(SWE_ERR_INVALID, "n must equal nx*nz");
  if (int rc = use_device(w)) return rc;
  SWE_CK(cudaMemcpyAsync(w->F.f[f], host, sizeof(float) * n, cudaMemcpyHostToDevice, w->stream));
  if (f == SWE_HEIGHT) {
    w->hq_valid = false;
    SWE_CK(cudaMemsetAsync(&w->cnt->exported_q, 0, sizeof(long long), w->stream));
  }
  SWE_CK(cudaStreamSynchronize(w->stream));
  return SWE_OK;
}

int swe_world_download(swe_world* w, swe_field f, float* host, size_t n) {
  if (!w || !host) return fail(SWE_ERR_INVALID, "NULL argument");
  if ((int)f < 0 || (int)f > 8) return fail(SWE_ERR_INVALID, "unknown field");
  if (n != (size_t)w->n) return fail(SWE_ERR_INVALID, "n must equal nx*nz");
  if (int rc = use_device(w)) return rc;
  SWE_CK(cudaMemcpyAsync(host, w->F.f[f], sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  return SWE_OK;
}

void swe_terrain_default(swe_terrain* t) {
  if (!t) return;
  std::memset(t, 0, sizeof(*t));
  t->octaves = 0;
  t->base_freq = 1.0f / 64.0f;
  t->lacunarity = 2.0f;
  t->persistence = 0.5f;
  t->top = 0.5f;
}

int swe_world_terrain(swe_world* w, const swe_terrain* t) {
  if (!w || !t) return fail(SWE_ERR_INVALID, "NULL argument");
  if (t->octaves < 0 || t->octaves > 32) return fail(SWE_ERR_INVALID, "octaves must be in [0, 32]");
  if (t->npyramids < 0 || (t->npyramids > 0 && !t->pyramids))
    return fail(SWE_ERR_INVALID, "npyramids must be >= 0 with a pyramid array");
  if (t->octaves > 0 && !(t->base_freq > 0.0f)) return fail(SWE_ERR_INVALID, "base_freq must be > 0");
  if (int rc = use_device(w)) return rc;
  swe::TerrainSpec ts;
  ts.seed = t->seed;
  ts.octaves = t->octaves;
  ts.base_freq = t->base_freq;
  ts.lacunarity = t->lacunarity;
  ts.persistence = t->persistence;
  ts.top = t->top;
  ts.sediment = t->sediment;
  ts.sediment_jitter = t->sediment_jitter;
  ts.npyramids = t->npyramids;
  ts.pyramids = t->pyramids;
  SWE_CK(swe::launch_terrain(w->F.f[SWE_HEIGHT], w->nx, w->nz, ts, w->stream));
  w->hq_valid = false;
  SWE_CK(cudaMemsetAsync(&w->cnt->exported_q, 0, sizeof(long long), w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  return SWE_OK;
}

int swe_world_device_field(swe_world* w, swe_field f, void** dev_ptr) {
  if (!w || !dev_ptr) return fail(SWE_ERR_INVALID, "NULL argument");
  if ((int)f < 0 || (int)f > 8) return fail(SWE_ERR_INVALID, "unknown field");
  *dev_ptr = w->F.f[f];
  return SWE_OK;
}

int swe_world_erode(swe_world* w, int cycles, int particles, swe_mode mode) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (cycles < 0 || particles < 0) return fail(SWE_ERR_INVALID, "cycles and particles must be >= 0");
  if (mode != SWE_MODE_ORDERED && mode != SWE_MODE_PARALLEL) return fail(SWE_ERR_INVALID, "unknown mode");
  if (int rc = use_device(w)) return rc;
  SWE_CK(cudaMemsetAsync(w->cnt, 0, 3 * sizeof(unsigned long long), w->stream));
  if (cycles == 0) return SWE_OK;
  const Consts c = w->consts();
  if (mode == SWE_MODE_ORDERED) {
    for (int k = 0; k < cycles; k++) {
      swe::launch_reset_tracks(w->F, w->n, w->stream);
      swe::launch_ordered_particles(w->F, c, w->grand, w->tape, w->tape_len, w->cnt, particles, w->stream);
      swe::launch_ema_float(w->F, c.lrate, w->n, w->stream);
    }
    SWE_CK(cudaGetLastError());
    w->hq_valid = false;
    return SWE_OK;
  }
  const int lanes = swe::par_lanes(w->p.lanes, w->nx, w->nz, particles);
  if (int rc = ensure_parallel(w, lanes)) return rc;
  if (int rc = clear_after_abort(w)) return rc;
  if (int rc = ensure_fixed(w)) return rc;
  SWE_CK(cudaMemsetAsync(&w->cnt->fly_ns, 0, 17 * sizeof(unsigned long long) + 8, w->stream));
  for (int k = 0; k < cycles; k++)
    if (int rc = enqueue_parallel_cycle(w, particles, lanes)) return rc;
  return SWE_OK;
}

int swe_world_set_wait_limit(swe_world* w, uint64_t ns) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  w->wait_ns = ns;
  return SWE_OK;
}

int swe_world_set_form(swe_world* w, int kind, int ctas) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (kind < 0 || kind > 3 || ctas < 0) return fail(SWE_ERR_INVALID, "kind must be 0, 1, 2 or 3 and ctas >= 0");
  w->form.kind = kind;
  w->form.ctas = ctas;
  return SWE_OK;
}

int swe_world_get_form(swe_world* w, int* kind, int* ctas) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (kind) *kind = w->form.kind;
  if (ctas) *ctas = w->form.ctas;
  return SWE_OK;
}

int swe_world_tune(swe_world* w, int particles, int* kind, int* ctas, double* best_ms, double* default_ms) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (particles < 1) return fail(SWE_ERR_INVALID, "particles must be >= 1");
  if (int rc = use_device(w)) return rc;
  const int lanes = swe::par_lanes(w->p.lanes, w->nx, w->nz, particles);
  char key[96];
  std::snprintf(key, sizeof key, "%dx%d:%d:%d", w->nx, w->nz, particles, lanes);
  if (best_ms) *best_ms = 0.0;
  if (default_ms) *default_ms = 0.0;
  {
    std::lock_guard<std::mutex> lock(g_form_mutex);
    auto it = g_forms.find(key);
    if (it != g_forms.end()) {
      w->form = it->second;
      if (kind) *kind = w->form.kind;
      if (ctas) *ctas = w->form.ctas;
      return SWE_OK;
    }
  }
  // A scratch world with this world's size, parameters, seed and heights.
  swe_world* r = nullptr;
  if (int rc = swe_world_create(w->nx, w->nz, &w->p, w->seed, &r)) return rc;
  int rc = SWE_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto done = [&](int code) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    swe_world_destroy(r);
    return code;
  };
  if (cudaMemcpyAsync(r->F.f[0], w->F.f[0], sizeof(float) * (size_t)w->n, cudaMemcpyDeviceToDevice, r->stream) !=
          cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return done(fail(SWE_ERR_CUDA, "setting up the launch-form tuner failed"));
  if ((rc = ensure_parallel(r, lanes)) != SWE_OK || (rc = ensure_fixed(r)) != SWE_OK) return done(rc);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, w->device);
  std::vector<swe::LaunchForm> cands;
  cands.push_back(swe::LaunchForm{0, 0});
  cands.push_back(swe::LaunchForm{1, 0});
  for (int div : {1, 2, 4}) cands.push_back(swe::LaunchForm{2, sms / div > 0 ? sms / div : 1});
  cands.push_back(swe::LaunchForm{2, 3 * sms / 4 > 0 ? 3 * sms / 4 : 1});
  for (int per = 2; per <= 4; per++) cands.push_back(swe::LaunchForm{2, per * sms});  // where they fit
  for (int per = 1; per <= 2; per++) cands.push_back(swe::LaunchForm{3, per * sms});  // lanes spread over 4 warps
  double best = -1.0;
  swe::LaunchForm best_form;
  for (size_t i = 0; i <= cands.size(); i++) {
    const swe::LaunchForm f = cands[i == 0 ? 0 : i - 1];  // the first form twice: a warm-up
    r->form = f;
    float ms = 0.0f;
    if (cudaEventRecord(e0, r->stream) != cudaSuccess) return done(fail(SWE_ERR_CUDA, "event record failed"));
    if ((rc = enqueue_parallel_cycle(r, particles, lanes)) != SWE_OK) return done(rc);
    if (cudaEventRecord(e1, r->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
      return done(fail(SWE_ERR_CUDA, "timing a launch form failed"));
    if (i == 0) continue;
    if (i == 1 && default_ms) *default_ms = ms;
    if (best < 0 || ms < best) {
      best = ms;
      best_form = f;
    }
  }
  uint32_t st = 0;
  if ((rc = swe_world_status(r, &st)) != SWE_OK) return done(rc);
  if (st) return done(fail(SWE_ERR_DEVICE, "a tuning cycle reported a device status"));
  {
    std::lock_guard<std::mutex> lock(g_form_mutex);
    g_forms[key] = best_form;
  }
  w->form = best_form;
  if (kind) *kind = best_form.kind;
  if (ctas) *ctas = best_form.ctas;
  if (best_ms) *best_ms = best;
  return done(SWE_OK);
}

int swe_world_get_cycle(swe_world* w, uint64_t* cycle) {
  if (!w || !cycle) return fail(SWE_ERR_INVALID, "NULL argument");
  if (int rc = use_device(w)) return rc;
  unsigned long long v = 0;
  SWE_CK(cudaMemcpyAsync(&v, &w->cnt->cycle, sizeof(v), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  *cycle = v;
  return SWE_OK;
}

int swe_world_set_cycle(swe_world* w, uint64_t cycle) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  const unsigned long long v = cycle;
  SWE_CK(cudaMemcpyAsync(&w->cnt->cycle, &v, sizeof(v), cudaMemcpyHostToDevice, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  return SWE_OK;
}

int swe_batch_erode(swe_world* const* worlds, int count, int cycles, const int* particles_per_cycle) {
  if (count < 0 || cycles < 0) return fail(SWE_ERR_INVALID, "count and cycles must be >= 0");
  if (count == 0) return SWE_OK;
  if (!worlds || !particles_per_cycle) return fail(SWE_ERR_INVALID, "NULL argument");
  for (int i = 0; i < count; i++) {
    if (!worlds[i]) return fail(SWE_ERR_INVALID, "a world is NULL");
    if (particles_per_cycle[i] < 0) return fail(SWE_ERR_INVALID, "particles_per_cycle must be >= 0");
    if (worlds[i]->device != worlds[0]->device) return fail(SWE_ERR_INVALID, "worlds on different devices");
  }
  {
    std::vector<swe_world*> sorted(worlds, worlds + count);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return fail(SWE_ERR_INVALID, "a world appears twice in the batch");
  }
  if (int rc = use_device(worlds[0])) return rc;
  std::vector<swe::BatchWorld> fit;
  std::vector<swe_world*> fit_w;
  for (int i = 0; i < count; i++) {
    swe_world* w = worlds[i];
    const int particles = particles_per_cycle[i];
    SWE_CK(cudaMemsetAsync(w->cnt, 0, 3 * sizeof(unsigned long long), w->stream));
    if (cycles == 0) continue;
    const int lanes = swe::par_lanes(w->p.lanes, w->nx, w->nz, particles);
    if (int rc = ensure_parallel(w, lanes)) return rc;
    if (int rc = clear_after_abort(w)) return rc;
    if (int rc = ensure_fixed(w)) return rc;
    SWE_CK(cudaMemsetAsync(&w->cnt->fly_ns, 0, 17 * sizeof(unsigned long long) + 8, w->stream));
    if (swe::batch_fits(lanes, w->nx, w->nz)) {
      swe::BatchWorld b;
      b.B = w->pb;
      b.F = w->F;
      b.c = w->consts();
      b.seed = w->seed;
      b.cnt = w->cnt;
      b.gb = w->gbar;
      b.particles = particles;
      b.lanes = lanes;
      fit.push_back(b);
      fit_w.push_back(w);
    } else {
      for (int k = 0; k < cycles; k++)
        if (int rc = enqueue_parallel_cycle(w, particles, lanes)) return rc;
    }
  }
  if (fit.empty()) return SWE_OK;
  // The persistent launch runs on the first batched world's stream, after
  // the work already queued on every batched world's stream.
  cudaStream_t s = fit_w[0]->stream;
  for (size_t i = 1; i < fit_w.size(); i++) {
    if (fit_w[i]->stream == s) continue;
    cudaEvent_t ev;
    SWE_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, fit_w[i]->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
    cudaEventDestroy(ev);
    SWE_CK(e);
  }
  SWE_CK(swe::launch_par_batch(fit.data(), (int)fit.size(), cycles, s));
  return SWE_OK;
}

}  // extern "C"

struct swe_batch {
  std::vector<swe_world*> worlds;
  std::vector<int> particles;
  std::vector<int> lanes;
  swe::BatchShape shape{16, 256};
  int clusters = 0;       // clusters launched for `shape`
  void* d_mem = nullptr;  // queue counter (first 256 bytes), then the world entries
  cudaStream_t stream = nullptr;
  int device = 0;
  double tuned_ms = 0.0, default_ms = 0.0;
};

namespace {

std::mutex g_tune_mutex;
std::map<std::string, swe::BatchShape> g_tuned;  // batch signature -> fastest shape

std::string batch_signature(const swe_batch& b) {
  std::vector<std::string> parts;
  for (size_t i = 0; i < b.worlds.size(); i++) {
    char buf[96];
    std::snprintf(buf, sizeof buf, "%dx%d:%d:%d", b.worlds[i]->nx, b.worlds[i]->nz, b.particles[i], b.lanes[i]);
    parts.emplace_back(buf);
  }
  std::sort(parts.begin(), parts.end());
  std::string key;
  for (auto& p : parts) key += p + ";";
  return key;
}

std::vector<swe::BatchWorld> batch_worlds(const std::vector<swe_world*>& ws, const std::vector<int>& particles,
                                          const std::vector<int>& lanes) {
  std::vector<swe::BatchWorld> out(ws.size());
  for (size_t i = 0; i < ws.size(); i++) {
    swe::BatchWorld& b = out[i];
    b.B = ws[i]->pb;
    b.F = ws[i]->F;
    b.c = ws[i]->consts();
    b.seed = ws[i]->seed;
    b.cnt = ws[i]->cnt;
    b.gb = ws[i]->gbar;
    b.particles = particles[i];
    b.lanes = lanes[i];
  }
  return out;
}

// Per world before a run: the tallies the world API resets per call, and the
// scratch an aborted cycle left behind.
int batch_prelude(swe_batch* b) {
  for (swe_world* w : b->worlds) {
    SWE_CK(cudaMemsetAsync(w->cnt, 0, 3 * sizeof(unsigned long long), b->stream));
    SWE_CK(cudaMemsetAsync(&w->cnt->fly_ns, 0, 17 * sizeof(unsigned long long) + 8, b->stream));
  }
  return SWE_OK;
}

// Times one cycle of shape `sh` on the scratch worlds `rep` (ms; < 0: the
// shape cannot run this batch).
double time_shape(swe_batch* b, const std::vector<swe_world*>& rep, const swe::BatchShape& sh, void* d_mem) {
  const int clusters = swe::batch_clusters(sh, (int)rep.size());
  if (clusters < 1) return -1.0;
  const std::vector<swe::BatchWorld> bw = batch_worlds(rep, b->particles, b->lanes);
  void* d_items = static_cast<char*>(d_mem) + 256;
  if (swe::upload_batch_items(bw.data(), (int)bw.size(), sh, d_items, b->stream) != cudaSuccess) {
    cudaGetLastError();
    return -1.0;
  }
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1.0;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return -1.0;
  }
  double ms = -1.0;
  cudaError_t e = cudaEventRecord(e0, b->stream);
  if (e == cudaSuccess)
    e = swe::launch_batch_items(d_items, static_cast<unsigned*>(d_mem), (int)bw.size(), 1, sh, clusters, b->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float f = 0.0f;
  if (e == cudaSuccess && cudaEventElapsedTime(&f, e0, e1) == cudaSuccess) ms = f;
  if (e != cudaSuccess) cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

// The autotuner: one cycle of every feasible shape on scratch copies of the
// worlds (same sizes, parameters, seeds and heights), fastest wins.
int tune_batch(swe_batch* b) {
  const std::string key = batch_signature(*b);
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      b->shape = it->second;
      return SWE_OK;
    }
  }
  std::vector<swe_world*> rep;
  auto cleanup = [&]() {
    for (swe_world* r : rep) swe_world_destroy(r);
  };
  for (size_t i = 0; i < b->worlds.size(); i++) {
    swe_world* w = b->worlds[i];
    swe_world* r = nullptr;
    int rc = swe_world_create(w->nx, w->nz, &w->p, w->seed, &r);
    if (rc != SWE_OK) {
      cleanup();
      return rc;
    }
    rep.push_back(r);
    // everything of the tuning runs on the batch's stream
    cudaStreamDestroy(r->stream);
    r->stream = b->stream;
    r->own_stream = false;
    if (cudaMemcpyAsync(r->F.f[0], w->F.f[0], sizeof(float) * (size_t)w->n, cudaMemcpyDeviceToDevice, b->stream) !=
        cudaSuccess) {
      cleanup();
      return fail(SWE_ERR_CUDA, "copying a height map for the autotuner failed");
    }
    if ((rc = ensure_parallel(r, b->lanes[i])) != SWE_OK || (rc = ensure_fixed(r)) != SWE_OK) {
      cleanup();
      return rc;
    }
  }
  static const swe::BatchShape kShapes[] = {{16, 256}, {16, 128}, {8, 256}, {8, 128}, {4, 256}, {4, 128}};
  double best = -1.0;
  swe::BatchShape best_shape{16, 256};
  time_shape(b, rep, kShapes[0], b->d_mem);  // warm-up: first launch of the kernel
  for (const swe::BatchShape& sh : kShapes) {
    const double ms = time_shape(b, rep, sh, b->d_mem);
    if (sh.ctas == 16 && sh.threads == 256) b->default_ms = ms > 0 ? ms : 0.0;
    if (ms > 0 && (best < 0 || ms < best)) {
      best = ms;
      best_shape = sh;
    }
  }
  cleanup();
  rep.clear();
  if (best < 0) return fail(SWE_ERR_CUDA, "no launch shape of the batch kernel can run this ensemble");
  b->shape = best_shape;
  b->tuned_ms = best;
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tuned[key] = best_shape;
  return SWE_OK;
}

}  // namespace

extern "C" {

int swe_batch_create(swe_world* const* worlds, int count, const int* particles_per_cycle, int tune, swe_batch** out) {
  if (!out) return fail(SWE_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (count < 1 || !worlds || !particles_per_cycle) return fail(SWE_ERR_INVALID, "a batch needs count >= 1 worlds");
  for (int i = 0; i < count; i++) {
    if (!worlds[i]) return fail(SWE_ERR_INVALID, "a world is NULL");
    if (particles_per_cycle[i] < 0) return fail(SWE_ERR_INVALID, "particles_per_cycle must be >= 0");
    if (worlds[i]->device != worlds[0]->device) return fail(SWE_ERR_INVALID, "worlds on different devices");
  }
  {
    std::vector<swe_world*> sorted(worlds, worlds + count);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return fail(SWE_ERR_INVALID, "a world appears twice in the batch");
  }
  if (int rc = use_device(worlds[0])) return rc;
  swe_batch* b = new swe_batch();
  b->device = worlds[0]->device;
  b->stream = worlds[0]->stream;
  auto bail = [&](int rc) {
    std::string msg = g_error;
    swe_batch_destroy(b);
    g_error = msg;
    return rc;
  };
  for (int i = 0; i < count; i++) {
    swe_world* w = worlds[i];
    const int lanes = swe::par_lanes(w->p.lanes, w->nx, w->nz, particles_per_cycle[i]);
    if (!swe::batch_fits(lanes, w->nx, w->nz))
      return bail(fail(SWE_ERR_INVALID, "a world has more particles in flight than one cluster holds (16,384)"));
    // everything queued on the worlds' own streams comes first
    if (cudaStreamSynchronize(w->stream) != cudaSuccess) return bail(fail(SWE_ERR_CUDA, "a world's stream failed"));
    if (int rc = ensure_parallel(w, lanes)) return bail(rc);
    if (int rc = clear_after_abort(w)) return bail(rc);
    if (int rc = ensure_fixed(w)) return bail(rc);
    if (cudaStreamSynchronize(w->stream) != cudaSuccess) return bail(fail(SWE_ERR_CUDA, "a world's stream failed"));
    b->worlds.push_back(w);
    b->particles.push_back(particles_per_cycle[i]);
    b->lanes.push_back(lanes);
  }
  if (cudaMalloc(&b->d_mem, 256 + swe::batch_item_bytes() * (size_t)count) != cudaSuccess) {
    cudaGetLastError();
    return bail(fail(SWE_ERR_NO_MEMORY, "cannot allocate the batch's device entries"));
  }
  if (tune)
    if (int rc = tune_batch(b)) return bail(rc);
  b->clusters = swe::batch_clusters(b->shape, count);
  if (b->clusters < 1) return bail(fail(SWE_ERR_CUDA, "the batch kernel cannot launch on this device"));
  const std::vector<swe::BatchWorld> bw = batch_worlds(b->worlds, b->particles, b->lanes);
  const cudaError_t e = swe::upload_batch_items(bw.data(), count, b->shape, static_cast<char*>(b->d_mem) + 256,
                                                b->stream);
  if (e != cudaSuccess) return bail(fail(SWE_ERR_CUDA, std::string("batch entries: ") + cudaGetErrorString(e)));
  *out = b;
  return SWE_OK;
}

int swe_batch_run(swe_batch* b, int cycles) {
  if (!b) return fail(SWE_ERR_INVALID, "NULL batch");
  if (cycles < 0) return fail(SWE_ERR_INVALID, "cycles must be >= 0");
  SWE_CK(cudaSetDevice(b->device));
  if (int rc = batch_prelude(b)) return rc;
  if (cycles == 0) return SWE_OK;
  for (swe_world* w : b->worlds) {
    if (w->scratch_dirty) {
      w->scratch_dirty = false;
      const size_t stride = ((size_t)w->n + 63) & ~(size_t)63;
      SWE_CK(cudaMemsetAsync(w->pb.dq, 0, sizeof(int32_t) * 4 * stride, b->stream));
    }
    if (!w->hq_valid) {
      swe::launch_height_to_fixed(w->F.f[0], w->pb.hq, w->consts(), w->cnt, b->stream);
      SWE_CK(cudaGetLastError());
      w->hq_valid = true;
    }
  }
  SWE_CK(swe::launch_batch_items(static_cast<char*>(b->d_mem) + 256, static_cast<unsigned*>(b->d_mem),
                                 (int)b->worlds.size(), cycles, b->shape, b->clusters, b->stream));
  return SWE_OK;
}

int swe_batch_shape(swe_batch* b, int* ctas_per_cluster, int* threads_per_cta, double* tuned_ms, double* default_ms) {
  if (!b) return fail(SWE_ERR_INVALID, "NULL batch");
  if (ctas_per_cluster) *ctas_per_cluster = b->shape.ctas;
  if (threads_per_cta) *threads_per_cta = b->shape.threads;
  if (tuned_ms) *tuned_ms = b->tuned_ms;
  if (default_ms) *default_ms = b->default_ms;
  return SWE_OK;
}

int swe_batch_set_shape(swe_batch* b, int ctas_per_cluster, int threads_per_cta) {
  if (!b) return fail(SWE_ERR_INVALID, "NULL batch");
  const swe::BatchShape sh{ctas_per_cluster, threads_per_cta};
  if (!swe::batch_shape_ok(sh))
    return fail(SWE_ERR_INVALID, "ctas_per_cluster must be 4, 8 or 16 and threads_per_cta a multiple of 32 up to 256");
  SWE_CK(cudaSetDevice(b->device));
  const int clusters = swe::batch_clusters(sh, (int)b->worlds.size());
  if (clusters < 1) return fail(SWE_ERR_INVALID, "this shape cannot launch");
  const std::vector<swe::BatchWorld> bw = batch_worlds(b->worlds, b->particles, b->lanes);
  const cudaError_t e = swe::upload_batch_items(bw.data(), (int)bw.size(), sh, static_cast<char*>(b->d_mem) + 256,
                                                b->stream);
  if (e == cudaErrorInvalidValue) return fail(SWE_ERR_INVALID, "a world's lanes do not fit one cluster of this shape");
  SWE_CK(e);
  b->shape = sh;
  b->clusters = clusters;
  return SWE_OK;
}

void swe_batch_destroy(swe_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  cudaFree(b->d_mem);
  delete b;
}

int swe_batch_erode_ordered(swe_world* const* worlds, int count, int cycles, const int* particles_per_cycle) {
  if (count < 0 || cycles < 0) return fail(SWE_ERR_INVALID, "count and cycles must be >= 0");
  if (count == 0) return SWE_OK;
  if (!worlds || !particles_per_cycle) return fail(SWE_ERR_INVALID, "NULL argument");
  for (int i = 0; i < count; i++) {
    if (!worlds[i]) return fail(SWE_ERR_INVALID, "a world is NULL");
    if (particles_per_cycle[i] < 0) return fail(SWE_ERR_INVALID, "particles_per_cycle must be >= 0");
    if (worlds[i]->device != worlds[0]->device) return fail(SWE_ERR_INVALID, "worlds on different devices");
  }
  {
    std::vector<swe_world*> sorted(worlds, worlds + count);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return fail(SWE_ERR_INVALID, "a world appears twice in the batch");
  }
  if (int rc = use_device(worlds[0])) return rc;
  // Everything runs on the first world's stream, after the work already
  // queued on the others' streams.
  cudaStream_t s = worlds[0]->stream;
  for (int i = 1; i < count; i++) {
    if (worlds[i]->stream == s) continue;
    cudaEvent_t ev;
    SWE_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, worlds[i]->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
    cudaEventDestroy(ev);
    SWE_CK(e);
  }
  std::vector<swe::OrderedWorld> items(count);
  long max_cells = 0;
  for (int i = 0; i < count; i++) {
    swe_world* w = worlds[i];
    SWE_CK(cudaMemsetAsync(w->cnt, 0, 3 * sizeof(unsigned long long), s));
    swe::OrderedWorld& o = items[i];
    o.F = w->F;
    o.c = w->consts();
    o.rng = w->grand;
    o.tape = w->tape;
    o.tape_len = w->tape_len;
    o.cnt = w->cnt;
    o.n = w->n;
    o.particles = particles_per_cycle[i];
    if (w->n > max_cells) max_cells = w->n;
  }
  int rc = SWE_OK;
  if (cycles > 0) {
    int sms = 0;
    SWE_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, worlds[0]->device));
    void* d = nullptr;
    SWE_CK(cudaMallocAsync(&d, sizeof(swe::OrderedWorld) * count, s));
    cudaError_t e = cudaMemcpyAsync(d, items.data(), sizeof(swe::OrderedWorld) * count, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = swe::launch_ordered_batch(static_cast<const swe::OrderedWorld*>(d), count, max_cells, cycles, sms, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = fail(SWE_ERR_CUDA, cudaGetErrorString(e));
  }
  for (int i = 0; i < count; i++) worlds[i]->hq_valid = false;
  return rc;
}

int swe_world_status(swe_world* w, uint32_t* status) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  SWE_CK(cudaStreamSynchronize(w->stream));
  unsigned int st = 0;
  SWE_CK(cudaMemcpy(&st, &w->cnt->status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st & SWE_STATUS_TIMEOUT) w->scratch_dirty = true;
  if (status) *status = st;
  return SWE_OK;
}

int swe_world_sync(swe_world* w) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  uint32_t st = 0;
  if (int rc = swe_world_status(w, &st)) return rc;
  if (st) {
    SWE_CK(cudaMemset(&w->cnt->status, 0, sizeof(unsigned int)));
    char buf[160];
    std::snprintf(buf, sizeof buf, "device status 0x%x:%s%s%s%s", st,
                  (st & SWE_STATUS_NONFINITE) ? " non-finite particle" : "",
                  (st & SWE_STATUS_RANGE) ? " fixed-point height out of range" : "",
                  (st & SWE_STATUS_TAPE) ? " rand tape exhausted" : "",
                  (st & SWE_STATUS_TIMEOUT) ? " a wait ran past its deadline (cycle aborted)" : "");
    return fail(SWE_ERR_DEVICE, buf);
  }
  return SWE_OK;
}

int swe_world_seed_rand(swe_world* w, uint32_t seed) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  GlibcRandState g;
  glibc_seed(g, seed);
  SWE_CK(cudaMemcpyAsync(w->grand, &g, sizeof(g), cudaMemcpyHostToDevice, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  return SWE_OK;
}

int swe_world_set_rand_tape(swe_world* w, const int32_t* tape, size_t n) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (n > 0 && !tape) return fail(SWE_ERR_INVALID, "tape is NULL");
  if (int rc = use_device(w)) return rc;
  SWE_CK(cudaStreamSynchronize(w->stream));
  if (w->tape) SWE_CK(cudaFree(w->tape));
  w->tape = nullptr;
  w->tape_len = 0;
  if (n > 0) {
    SWE_CK(cudaMalloc(&w->tape, sizeof(int32_t) * n));
    SWE_CK(cudaMemcpy(w->tape, tape, sizeof(int32_t) * n, cudaMemcpyHostToDevice));
    w->tape_len = (long long)n;
  }
  SWE_CK(cudaMemset(&w->cnt->tape_pos, 0, sizeof(long long)));
  return SWE_OK;
}

int swe_world_mass_ledger(swe_world* w, int64_t* map_q, int64_t* inflight_q, int64_t* exported_q) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  if (int rc = ensure_parallel(w, 0)) return rc;
  if (int rc = ensure_fixed(w)) return rc;
  SWE_CK(cudaMemsetAsync(w->dsum, 0, sizeof(long long), w->stream));
  swe::launch_sum_fixed(w->pb.hq, w->n, w->dsum, w->stream);
  SWE_CK(cudaGetLastError());
  long long s = 0, e = 0;
  SWE_CK(cudaMemcpyAsync(&s, w->dsum, sizeof(s), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaMemcpyAsync(&e, &w->cnt->exported_q, sizeof(e), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  if (map_q) *map_q = s;
  if (inflight_q) *inflight_q = 0;
  if (exported_q) *exported_q = e;
  return SWE_OK;
}

int swe_world_stats(swe_world* w, int64_t* particle_steps, int64_t* particles, int64_t* transfers) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  unsigned long long v[3] = {0, 0, 0};
  SWE_CK(cudaMemcpyAsync(v, w->cnt, sizeof(v), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  if (particle_steps) *particle_steps = (int64_t)v[0];
  if (particles) *particles = (int64_t)v[1];
  if (transfers) *transfers = (int64_t)v[2];
  return SWE_OK;
}

int swe_trace_particles(swe_world* w, const float* spawn_xz, int n, int steps, const int32_t* turb_tape,
                        float* out_state) {
  if (!w || !spawn_xz || !turb_tape || !out_state) return fail(SWE_ERR_INVALID, "NULL argument");
  if (n < 0 || steps < 0) return fail(SWE_ERR_INVALID, "n and steps must be >= 0");
  if (n == 0 || steps == 0) return SWE_OK;
  if (int rc = use_device(w)) return rc;
  const size_t nrec = (size_t)n * steps;
  float* d_spawn = nullptr;
  int32_t* d_tape = nullptr;
  float* d_out = nullptr;
  int rc = SWE_OK;
  auto run = [&]() -> int {
    SWE_CK(cudaMalloc(&d_spawn, sizeof(float) * 2 * n));
    SWE_CK(cudaMalloc(&d_tape, sizeof(int32_t) * 3 * nrec));
    SWE_CK(cudaMalloc(&d_out, sizeof(float) * 9 * nrec));
    SWE_CK(cudaMemcpyAsync(d_spawn, spawn_xz, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, w->stream));
    SWE_CK(cudaMemcpyAsync(d_tape, turb_tape, sizeof(int32_t) * 3 * nrec, cudaMemcpyHostToDevice, w->stream));
    swe::launch_trace(w->F.f[0], w->consts(), d_spawn, n, steps, d_tape, d_out, w->stream);
    SWE_CK(cudaGetLastError());
    SWE_CK(cudaMemcpyAsync(out_state, d_out, sizeof(float) * 9 * nrec, cudaMemcpyDeviceToHost, w->stream));
    SWE_CK(cudaStreamSynchronize(w->stream));
    return SWE_OK;
  };
  rc = run();
  cudaFree(d_spawn);
  cudaFree(d_tape);
  cudaFree(d_out);
  return rc;
}

int swe_world_fly(swe_world* w, float x, float z, int steps, const int32_t* turb_tape, float* out_state,
                  int* ok_steps) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (steps < 0) return fail(SWE_ERR_INVALID, "steps must be >= 0");
  if (int rc = use_device(w)) return rc;
  int32_t* d_tape = nullptr;
  float* d_out = nullptr;
  int* d_ok = nullptr;
  auto run = [&]() -> int {
    if (turb_tape && steps > 0) {
      SWE_CK(cudaMalloc(&d_tape, sizeof(int32_t) * 3 * (size_t)steps));
      SWE_CK(cudaMemcpyAsync(d_tape, turb_tape, sizeof(int32_t) * 3 * (size_t)steps, cudaMemcpyHostToDevice,
                             w->stream));
    }
    if (out_state && steps > 0) SWE_CK(cudaMalloc(&d_out, sizeof(float) * 9 * (size_t)steps));
    SWE_CK(cudaMalloc(&d_ok, sizeof(int)));
    swe::launch_fly_live(w->F, w->consts(), x, z, steps, d_tape, w->grand, d_out, d_ok, w->cnt, w->stream);
    SWE_CK(cudaGetLastError());
    if (d_out)
      SWE_CK(cudaMemcpyAsync(out_state, d_out, sizeof(float) * 9 * (size_t)steps, cudaMemcpyDeviceToHost,
                             w->stream));
    int ok = 0;
    SWE_CK(cudaMemcpyAsync(&ok, d_ok, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    SWE_CK(cudaStreamSynchronize(w->stream));
    if (ok_steps) *ok_steps = ok;
    return SWE_OK;
  };
  int rc = run();
  cudaFree(d_tape);
  cudaFree(d_out);
  cudaFree(d_ok);
  w->hq_valid = false;
  return rc;
}

int swe_world_cascade_at(swe_world* w, int x, int z) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (x < 0 || z < 0 || x >= w->nx || z >= w->nz) return fail(SWE_ERR_INVALID, "cell out of bounds");
  if (int rc = use_device(w)) return rc;
  swe::launch_cascade_at(w->F.f[0], w->consts(), x, z, w->stream);
  SWE_CK(cudaGetLastError());
  SWE_CK(cudaStreamSynchronize(w->stream));
  w->hq_valid = false;
  return SWE_OK;
}

int swe_world_normals(swe_world* w, float* host_out, size_t n) {
  if (!w || !host_out) return fail(SWE_ERR_INVALID, "NULL argument");
  if (n != 3 * (size_t)w->n) return fail(SWE_ERR_INVALID, "n must equal 3*nx*nz");
  if (int rc = use_device(w)) return rc;
  float* d_out = nullptr;
  auto run = [&]() -> int {
    SWE_CK(cudaMalloc(&d_out, sizeof(float) * n));
    swe::launch_normals(w->F.f[0], w->consts(), d_out, w->stream);
    SWE_CK(cudaGetLastError());
    SWE_CK(cudaMemcpyAsync(host_out, d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream));
    SWE_CK(cudaStreamSynchronize(w->stream));
    return SWE_OK;
  };
  int rc = run();
  cudaFree(d_out);
  return rc;
}

int swe_world_vertices(swe_world* w, float* host_out, size_t n) {
  if (!w || !host_out) return fail(SWE_ERR_INVALID, "NULL argument");
  if (n != 12 * (size_t)w->n) return fail(SWE_ERR_INVALID, "n must equal 12*nx*nz");
  if (int rc = use_device(w)) return rc;
  float* d_out = nullptr;
  auto run = [&]() -> int {
    SWE_CK(cudaMallocAsync(&d_out, sizeof(float) * n, w->stream));
    swe::launch_vertices(w->F.f[0], w->consts(), d_out, w->stream);
    SWE_CK(cudaGetLastError());
    SWE_CK(cudaMemcpyAsync(host_out, d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream));
    SWE_CK(cudaStreamSynchronize(w->stream));
    return SWE_OK;
  };
  int rc = run();
  if (d_out) cudaFreeAsync(d_out, w->stream);
  return rc;
}

int swe_world_windmap(swe_world* w, float* host_rgba, size_t n) {
  if (!w || !host_rgba) return fail(SWE_ERR_INVALID, "NULL argument");
  if (n != 4 * (size_t)w->n) return fail(SWE_ERR_INVALID, "n must equal 4*nx*nz");
  if (int rc = use_device(w)) return rc;
  float* d_out = nullptr;
  auto run = [&]() -> int {
    SWE_CK(cudaMallocAsync(&d_out, sizeof(float) * n, w->stream));
    swe::launch_windmap(w->F, w->n, d_out, w->stream);
    SWE_CK(cudaGetLastError());
    SWE_CK(cudaMemcpyAsync(host_rgba, d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream));
    SWE_CK(cudaStreamSynchronize(w->stream));
    return SWE_OK;
  };
  int rc = run();
  if (d_out) cudaFreeAsync(d_out, w->stream);
  return rc;
}

int swe_world_get_stream(swe_world* w, void** stream) {
  if (!w || !stream) return fail(SWE_ERR_INVALID, "NULL argument");
  *stream = (void*)w->stream;
  return SWE_OK;
}

int swe_world_set_stream(swe_world* w, void* stream) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  SWE_CK(cudaStreamSynchronize(w->stream));
  if (w->own_stream) SWE_CK(cudaStreamDestroy(w->stream));
  if (stream) {
    w->stream = (cudaStream_t)stream;
    w->own_stream = false;
  } else {
    SWE_CK(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
    w->own_stream = true;
  }
  return SWE_OK;
}

int swe_world_kernel_times(swe_world* w, double* fly_ms, double* cascade_ms) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  unsigned long long t[2] = {0, 0};
  SWE_CK(cudaMemcpyAsync(t, &w->cnt->fly_ns, sizeof(t), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  if (fly_ms) *fly_ms = (double)t[0] * 1e-6;
  if (cascade_ms) *cascade_ms = (double)t[1] * 1e-6;
  return SWE_OK;
}

int swe_world_phase_times(swe_world* w, double* ms, int n) {
  if (!w || !ms) return fail(SWE_ERR_INVALID, "NULL argument");
  if (n < 0 || n > 13) return fail(SWE_ERR_INVALID, "n must be in [0, 13]");
  if (int rc = use_device(w)) return rc;
  unsigned long long t[13];
  SWE_CK(cudaMemcpyAsync(t, w->cnt->phase_ns, sizeof(t), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  for (int k = 0; k < n; k++) ms[k] = (double)t[k] * 1e-6;
  return SWE_OK;
}

int swe_world_cascade_stats(swe_world* w, int64_t* cascades, int64_t* cells, int* max_iters) {
  if (!w) return fail(SWE_ERR_INVALID, "NULL world");
  if (int rc = use_device(w)) return rc;
  unsigned long long v[2] = {0, 0};
  unsigned int m = 0;
  SWE_CK(cudaMemcpyAsync(v, &w->cnt->cascades, sizeof(v), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaMemcpyAsync(&m, &w->cnt->max_cascade_iters, sizeof(m), cudaMemcpyDeviceToHost, w->stream));
  SWE_CK(cudaStreamSynchronize(w->stream));
  if (cascades) *cascades = (int64_t)v[0];
  if (cells) *cells = (int64_t)v[1];
  if (max_iters) *max_iters = (int)m;
  return SWE_OK;
}

int swe_world_expf_bits(swe_world* w, uint32_t first_bits, size_t n, float* host_y) {
  if (!w || !host_y) return fail(SWE_ERR_INVALID, "NULL argument");
  if (n == 0) return SWE_OK;
  if ((uint64_t)first_bits + n > (1ull << 32)) return fail(SWE_ERR_INVALID, "bit range exceeds 32 bits");
  if (int rc = use_device(w)) return rc;
  float* d_out = nullptr;
  auto run = [&]() -> int {
    SWE_CK(cudaMalloc(&d_out, sizeof(float) * n));
    swe::launch_expf_bits(w->consts(), first_bits, (long)n, d_out, w->stream);
    SWE_CK(cudaGetLastError());
    SWE_CK(cudaMemcpyAsync(host_y, d_out, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream));
    SWE_CK(cudaStreamSynchronize(w->stream));
    return SWE_OK;
  };
  int rc = run();
  cudaFree(d_out);
  return rc;
}

}  // extern "C"
