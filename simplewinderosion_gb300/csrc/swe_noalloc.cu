// Parallel erosion for callers that cannot allocate device memory.
//
// Some hosts of this code may not call cudaMalloc: a frame loop embedded in a
// render or game engine that owns the GPU's memory pool (the reference's own
// app erodes once per rendered frame, SimpleWindErosion.cpp:212-231), or code
// running while another framework's allocator owns the device memory. They
// still own the nine cell fields (inputs and outputs), but not the scratch
// the parallel kernel needs: fixed-point maps, track accumulators, counters
// and the grid barrier (particle state stays in shared memory: the call
// takes only the bounded-lanes kernel forms). swe_erode_parallel_noalloc
// keeps that scratch in one file-scope device array of fixed size, so it
// allocates nothing; every GPU that loads the library holds the array until
// the process exits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "swe.h"
#include "swe_kernels.h"

namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr size_t kMaxCells = SWE_NOALLOC_MAX_CELLS;          // a multiple of 64
constexpr size_t kMaxParticles = SWE_NOALLOC_MAX_PARTICLES;
constexpr size_t kCountersBytes = align256(sizeof(swe::Counters));
constexpr size_t kBarrierBytes = align256(sizeof(swe::GridBarrier));
constexpr size_t kBitWords = ((kMaxCells + 128) / 32 + 2 + 63) & ~(size_t)63;  // one visited bitmap
// heights; deltas, owed cascades, owners of even and odd steps; 3 bitmaps
constexpr size_t kMapsBytes = (7 * kMaxCells + 3 * kBitWords) * sizeof(int32_t);
constexpr size_t kTracksBytes = 4 * kMaxCells * sizeof(long long);   // track accumulators
constexpr size_t kWordsBytes = (kMaxCells + 32) * sizeof(unsigned long long);  // height words + padding
constexpr size_t kScratchBytes = kCountersBytes + kBarrierBytes + kMapsBytes + kTracksBytes + kWordsBytes;

// The scratch. In host code this name is only a stand-in for the device
// object: its device address comes from cudaGetSymbolAddress, per device.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct DeviceScratch {
  unsigned char* base = nullptr;  // device address of g_scratch on this device
  int grid = 0;                   // co-resident blocks of the cycle kernel
  bool ready = false;
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
DeviceScratch g_devices[kMaxDevices];

// Messages go to the same per-thread slot swe_last_error() reads.
int fail(int code, const std::string& msg) {
  swe::set_last_error(msg);
  return code;
}

// Once per device, with that device current: the device address of the
// scratch array and the launch size of the cycle kernel.
int setup_device(int dev, DeviceScratch** out) {
  if (dev < 0 || dev >= kMaxDevices) return fail(SWE_ERR_INVALID, "device index beyond the no-alloc table");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceScratch& d = g_devices[dev];
  if (!d.ready) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return fail(SWE_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    const int grid = swe::cycle_grid(dev);
    if (grid < 1) return fail(SWE_ERR_CUDA, "device cannot run the cooperative cycle kernel");
    d.base = static_cast<unsigned char*>(p);
    d.grid = grid;
    d.ready = true;
  }
  *out = &d;
  return SWE_OK;
}

}  // namespace

#define SWE_NA_CK(call)                                                                            \
  do {                                                                                             \
    const cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return fail(SWE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

extern "C" int swe_erode_parallel_noalloc(float* const* fields, int nx, int nz, const swe_params* p,
                                          uint64_t seed, uint64_t first_cycle, int cycles,
                                          int particles_per_cycle, void* stream, uint32_t* status) {
  if (!fields || !p) return fail(SWE_ERR_INVALID, "NULL argument");
  for (int k = 0; k < 9; k++)
    if (!fields[k]) return fail(SWE_ERR_INVALID, "a field pointer is NULL");
  if (nx < 1 || nz < 1) return fail(SWE_ERR_INVALID, "nx and nz must be >= 1");
  if ((size_t)nx * (size_t)nz > kMaxCells)
    return fail(SWE_ERR_INVALID, "nx*nz exceeds SWE_NOALLOC_MAX_CELLS (262144) of the static scratch");
  if (particles_per_cycle < 0 || (size_t)particles_per_cycle > kMaxParticles)
    return fail(SWE_ERR_INVALID, "particles_per_cycle must be in [0, SWE_NOALLOC_MAX_PARTICLES (65536)]");
  if (cycles < 0) return fail(SWE_ERR_INVALID, "cycles must be >= 0");
  if (p->max_age < 0 || p->max_age > 1000000) return fail(SWE_ERR_INVALID, "max_age must be in [0, 1e6]");
  if (p->frac_bits < 8 || p->frac_bits > 28) return fail(SWE_ERR_INVALID, "frac_bits must be in [8, 28]");
  if (!(p->boundarylayer != 0.0f)) return fail(SWE_ERR_INVALID, "boundarylayer must be non-zero");

  int dev = 0;
  SWE_NA_CK(cudaGetDevice(&dev));
  DeviceScratch* ds = nullptr;
  if (int rc = setup_device(dev, &ds)) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const long n = (long)nx * nz;
  const size_t stride = ((size_t)n + 63) & ~(size_t)63;
  const int lanes = swe::par_lanes(p->lanes, nx, nz, particles_per_cycle);
  // Particles in flight live in the bounded-lanes kernel's shared memory;
  // the all-at-once kernel would need particle buffers this call lacks.
  if (!swe::lanes_form_fits(lanes, n))
    return fail(SWE_ERR_INVALID, "more particles in flight than the bounded-lanes kernel holds on this GPU");
  unsigned char* base = ds->base;
  swe::Counters* cnt = reinterpret_cast<swe::Counters*>(base);
  swe::GridBarrier* gb = reinterpret_cast<swe::GridBarrier*>(base + kCountersBytes);
  int32_t* maps = reinterpret_cast<int32_t*>(base + kCountersBytes + kBarrierBytes);
  long long* tracks = reinterpret_cast<long long*>(base + kCountersBytes + kBarrierBytes + kMapsBytes);
  unsigned long long* words =
      reinterpret_cast<unsigned long long*>(base + kCountersBytes + kBarrierBytes + kMapsBytes + kTracksBytes);

  swe::ParallelBuffers B{};
  B.hq = maps;
  B.dq = maps + stride;
  B.visits = maps + 2 * stride;
  B.dq2 = maps + 3 * stride;
  B.visits2 = maps + 4 * stride;
  B.owner = maps + 5 * stride;
  B.owner2 = maps + 6 * stride;
  for (int k = 0; k < 3; k++) B.vbits[k] = reinterpret_cast<uint32_t*>(maps + 7 * stride + k * kBitWords);
  B.vbits_words = (long)((n + 128) / 32 + 2);
  B.hw = words + 1;  // one padding word before (and after) the map
  for (int k = 0; k < 4; k++) B.tq[k] = tracks + (size_t)k * n;
  B.capacity = 0;  // no particle buffers (B.state stays null)

  swe::Fields F;
  for (int k = 0; k < 9; k++) F.f[k] = fields[k];

  swe::Consts c{};
  c.nx = nx;
  c.nz = nz;
  c.max_age = p->max_age;
  c.boundarylayer = p->boundarylayer;
  c.suspension = p->suspension;
  c.gravity = p->gravity;
  c.lrate = p->lrate;
  c.maxdiff = p->maxdiff;
  c.settling = p->settling;
  c.mapscale = p->mapscale;
  c.px = p->pspeed[0];
  c.py = p->pspeed[1];
  c.pz = p->pspeed[2];
  c.frac_bits = p->frac_bits;
  c.scale = (float)(1u << p->frac_bits);
  c.inv_scale = 1.0f / c.scale;

  // The array keeps the last call's contents: reset everything a cycle
  // expects at zero, then set the random-number cycle counter (by a kernel
  // argument, so nothing is read from host memory later).
  SWE_NA_CK(cudaMemsetAsync(cnt, 0, sizeof(swe::Counters), s));
  swe::launch_set_cycle(cnt, first_cycle, s);
  SWE_NA_CK(cudaMemsetAsync(B.dq, 0, 2 * stride * sizeof(int32_t), s));
  SWE_NA_CK(cudaMemsetAsync(B.dq2, 0, 2 * stride * sizeof(int32_t), s));
  swe::launch_height_to_fixed(F.f[0], B.hq, c, cnt, s);
  SWE_NA_CK(cudaGetLastError());
  for (int k = 0; k < cycles; k++) {
    SWE_NA_CK(cudaMemsetAsync(gb, 0, sizeof(swe::GridBarrier), s));
    SWE_NA_CK(swe::launch_par_cycle(B, F, c, seed, cnt, gb, particles_per_cycle, lanes, ds->grid, s));
  }
  if (status) {
    SWE_NA_CK(cudaStreamSynchronize(s));
    uint32_t st = 0;
    SWE_NA_CK(cudaMemcpy(&st, &cnt->status, sizeof(st), cudaMemcpyDeviceToHost));
    *status = st;
    if (st) return fail(SWE_ERR_DEVICE, "device status bits set (see SWE_STATUS_*)");
  }
  return SWE_OK;
}
