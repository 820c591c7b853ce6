// Host-side launchers of the erosion kernels (internal to the library).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "swe_types.h"

namespace swe {

// Nine float fields in quad::cell order (cellpool.h:226-240).
struct Fields {
  float* f[9];
};

// The calling thread's error message, read by swe_last_error (swe_capi.cu).
void set_last_error(const std::string& msg);

// ---- exact modes (swe_exact.cu) ----
void launch_reset_tracks(const Fields& F, long n, cudaStream_t s);
void launch_ema_float(const Fields& F, float lrate, long n, cudaStream_t s);
void launch_ordered_particles(const Fields& F, const Consts& c, GlibcRandState* rng, const int32_t* tape,
                              long long tape_len, Counters* cnt, int particles, cudaStream_t s);
// One world of an ORDERED ensemble (launch_ordered_batch).
struct OrderedWorld {
  Fields F;
  Consts c;
  GlibcRandState* rng;
  const int32_t* tape;  // nullptr: the rand() replica
  long long tape_len;
  Counters* cnt;
  long n;         // cells
  int particles;  // per cycle
};
// `cycles` ORDERED erode cycles of every world of the device array `worlds`
// on stream s: per cycle all worlds' tracks are reset, each world's
// particles run in order on one thread of its own, then the fields take
// their update. max_cells: the largest world's cells; sms: the device's SMs.
cudaError_t launch_ordered_batch(const OrderedWorld* worlds, int count, long max_cells, int cycles, int sms,
                                 cudaStream_t s);
void launch_trace(const float* height, const Consts& c, const float* spawn_xz, int n, int steps,
                  const int32_t* tape, float* out, cudaStream_t s);
void launch_fly_live(const Fields& F, const Consts& c, float x, float z, int steps, const int32_t* tape,
                     GlibcRandState* rng, float* out, int* ok_steps, Counters* cnt, cudaStream_t s);
void launch_cascade_at(float* height, const Consts& c, int x, int z, cudaStream_t s);
void launch_normals(const float* height, const Consts& c, float* out, cudaStream_t s);
void launch_expf_bits(const Consts& c, uint32_t first, long n, float* out, cudaStream_t s);

// ---- parallel fixed-point mode (swe_parallel.cu) ----
struct ParallelBuffers {
  int32_t* hq;         // fixed-point heights
  int32_t* dq;         // exchange deltas pending for the cascade passes (zero between steps)
  int32_t* visits;     // cascades owed per cell (zero between steps)
  // bounded-lanes form: the maps of odd steps (the even steps use dq and
  // visits), so that a step's flights can start while the previous step's
  // last cascades finish
  int32_t* dq2;
  int32_t* visits2;
  int32_t* owner;      // the lowest lane id among a step's visitors of the cell (0x7FFFFFFF: none)
  int32_t* owner2;
  uint32_t* vbits[3];  // visited bitmaps of steps 0, 1, 2 mod 3 (cell i: bit 64 + i)
  long vbits_words;    // words in each bitmap, (n + 128) / 32 + 2
  unsigned long long* hw;  // height words (fixed-point height, write tag); hw[-1] and hw[n] exist (padding)
  long long* tq[4];    // track accumulators (massflow, momx, momy, momz), 2^-32 units
  ParticleSoA state[2];
  int capacity;        // particles the state buffers hold
};

void launch_height_to_fixed(const float* height, int32_t* q, const Consts& c, Counters* cnt, cudaStream_t s);
// Number of co-resident blocks of the persistent cycle kernel (0 if the
// device cannot launch cooperative kernels).
int cycle_grid(int device);
// Launch form of a bounded-lanes cycle: kind 0 the default rule (one 16-CTA
// cluster up to 4,096 lanes, else one CTA per SM), 1 one cluster (up to
// 16,384 lanes), 2 a cooperative grid of `ctas` CTAs (0: one per SM), 3 the
// same with 128 threads per CTA and the CTA's lanes spread over its four
// warps (fewer lanes per warp, so a warp's polling loops wait on fewer
// cells). The form changes no result: only the set of particles in flight
// matters.
struct LaunchForm {
  int kind = 0;
  int ctas = 0;
};
// One parallel erode cycle as one cooperative kernel.
cudaError_t launch_par_cycle(const ParallelBuffers& B, const Fields& F, const Consts& c, uint64_t seed,
                             Counters* cnt, GridBarrier* gb, int particles, int lanes, int grid, cudaStream_t s,
                             const LaunchForm& form = LaunchForm());
// Whether `lanes` particles in flight on an n-cell map take the bounded-lanes
// kernel (one 16-CTA cluster, or one CTA per SM), whose particle state lives
// in shared memory; otherwise launch_par_cycle needs B.state to hold them.
bool lanes_form_fits(int lanes, long n);
// Sets the cycle counter (which keys the parallel mode's random numbers) on
// the device, in stream order.
void launch_set_cycle(Counters* cnt, uint64_t cycle, cudaStream_t s);
// Particles in flight at once: lanes > 0 as given, 0 -> max(1024, cells/256),
// < 0 -> all particles of the cycle; never more than the cycle's particles.
int par_lanes(int lanes, int nx, int nz, int particles);
void launch_sum_fixed(const int32_t* hq, long n, long long* out, cudaStream_t s);

// ---- observables (swe_export.cu) ----
// RGBA wind map of the momentum fields into out_rgba (4*n floats, device,
// 16-byte aligned).
void launch_windmap(const Fields& F, long n, float* out_rgba, cudaStream_t s);
// Surface vertices of updatenode: 12 floats per cell (P, N, T-P, B-P).
void launch_vertices(const float* height, const Consts& c, float* out, cudaStream_t s);

// ---- initial terrains (swe_terrain.cu) ----
struct TerrainSpec {
  uint64_t seed;
  int octaves;  // 0: the reference's Gaussian bump
  double base_freq, lacunarity, persistence, top, sediment, sediment_jitter;
  int npyramids;
  const float* pyramids;  // host, npyramids x (cx, cz, height, base)
};
// Writes the terrain to `height` (nx*nz floats on the device); returns after
// it is done.
cudaError_t launch_terrain(float* height, int nx, int nz, const TerrainSpec& t, cudaStream_t s);

// One world of an ensemble run by launch_par_batch.
struct BatchWorld {
  ParallelBuffers B;
  Fields F;
  Consts c;
  uint64_t seed;
  Counters* cnt;
  GridBarrier* gb;
  int particles;  // per cycle
  int lanes;      // particles in flight (par_lanes)
};
// Whether a world with `lanes` in flight fits one 16-CTA cluster of the batch kernel.
bool batch_fits(int lanes, int nx, int nz);
// `cycles` parallel erode cycles of every world in one persistent launch of
// 16-CTA clusters on stream s (the worlds' height maps already in fixed
// point). Returns after the launch has completed.
cudaError_t launch_par_batch(const BatchWorld* worlds, int count, int cycles, cudaStream_t s);
// Launch shape of the batch kernel: CTAs per cluster (4, 8 or 16; one world
// per cluster at a time) and threads per CTA (a multiple of 32 up to 256).
// It changes no result: a world's lanes are spread over its cluster's
// threads, and only the set of particles in flight matters.
struct BatchShape {
  int ctas;
  int threads;
};
bool batch_shape_ok(const BatchShape& sh);
// Bytes of one world's entry in the device array of a prepared batch.
size_t batch_item_bytes();
// Writes the entries of `count` worlds for shape `sh` to d_items (device,
// count * batch_item_bytes()); returns after the copy. cudaErrorInvalidValue
// if a world's lanes do not fit one cluster of that shape.
cudaError_t upload_batch_items(const BatchWorld* worlds, int count, const BatchShape& sh, void* d_items,
                               cudaStream_t s);
// Clusters of shape `sh` to launch for a batch of `count` worlds: those that
// run at once, at most `count` (0: the shape cannot launch). Also sets the
// kernel's launch attributes, so call it before launch_batch_items.
int batch_clusters(const BatchShape& sh, int count);
// `cycles` cycles of a prepared batch on `clusters` clusters: resets the
// queue counter (d_queue, device) and launches the persistent kernel on s.
// Only a memset and a kernel launch are enqueued, so it can be captured into
// a CUDA graph.
cudaError_t launch_batch_items(const void* d_items, unsigned* d_queue, int count, int cycles, const BatchShape& sh,
                               int clusters, cudaStream_t s);

// ---- learned surrogate building blocks (swe_surrogate.cu): bf16 NHWC ----
cudaError_t nn_conv3x3(const void* x, const void* w, const float* bias, void* y, int N, int H, int W, int cin,
                       int cout, cudaStream_t s);
cudaError_t nn_flip(const void* w, void* wf, int cin, int cout, cudaStream_t s);
cudaError_t nn_conv_wgrad(const void* x, const void* dy, float* dw, float* db, int N, int H, int W, int cin, int cout,
                          cudaStream_t s);
cudaError_t nn_gelu(const void* pre, void* act, long n, cudaStream_t s);
// db (fp32 [cout]) += sum over the M pixels of dy (bf16 [M, cout]).
cudaError_t nn_bias_grad(const void* dy, float* db, long M, int cout, cudaStream_t s);
cudaError_t nn_gelu_bwd(const void* pre, const void* dact, void* dpre, long n, cudaStream_t s);
cudaError_t nn_pool2(const void* x, void* y, int N, int H, int W, int C, bool backward, cudaStream_t s);
cudaError_t nn_up2(const void* x, void* y, int N, int H, int W, int C, bool backward, cudaStream_t s);
cudaError_t nn_add(const void* a, const void* b, void* out, long n, cudaStream_t s);
// means (device, N floats) or nullptr: each map's mean, written first, and
// the heights moved so that the mean is ref
cudaError_t nn_pack_input(const float* h, const float* wind_xz, void* x, int N, int H, int W, cudaStream_t s,
                          float* means, float ref);
cudaError_t nn_mse(const void* pred, const float* target, float tscale, void* dpred, float* loss, long M, int C,
                   float gscale, cudaStream_t s);
cudaError_t nn_channel0(const void* pred, float* out, long M, int C, float oscale, cudaStream_t s);
cudaError_t nn_adam(float* w, const float* grad, float* m, float* v, void* w16, long n, float lr, float b1, float b2,
                    float eps, int step, cudaStream_t s);
cudaError_t nn_to_bf16(const float* a, void* b, long n, cudaStream_t s);
// ---- tensor-core (tcgen05/TMEM/TMA) convolutions (swe_umma.cu) ----
bool nn_conv_tc_supported(int H, int W, int kc, int nc);
cudaError_t nn_pack_tc(const void* w, void* wp, int cin, int cout, bool flip, cudaStream_t s);
cudaError_t nn_conv_tc(const void* x, const void* wp, const float* bias, void* y, void* act, int N, int H, int W,
                       int kc, int nc, cudaStream_t s);
bool nn_wgrad_tc_supported(int H, int W, int cin, int cout);
// dw (fp32 [cout,3,3,cin]) += the weight gradient, and db (fp32 [cout], or
// nullptr) += the bias gradient; sms: the device's SMs (sizes the split over pixels).
cudaError_t nn_wgrad_tc(const void* x, const void* dy, float* dw, float* db, int N, int H, int W, int cin, int cout,
                        int sms, cudaStream_t s);
// The first error code a tensor-core kernel recorded since the last call (0: none); clears it.
cudaError_t nn_tc_status(unsigned int* code);

}  // namespace swe
