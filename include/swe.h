/*
 * swe.h — C ABI of the GB300 SimpleWindErosion hot path.
 *
 * Drop-in for the reference's static simulation API (source/world.hpp:9-24,
 * source/wind.hpp:4-21): World::erode(int) and the World/Wind statics become
 * a world object with device-resident cell maps. The reference has no FFI;
 * each entry point below names the reference interface it replaces.
 *
 * Conventions
 *  - Return value: SWE_OK (0) or a negative SWE_ERR_* code; swe_last_error()
 *    gives the message of the calling thread's last failure.
 *  - Ownership: the caller owns host buffers; the library owns device memory.
 *  - Threading: one world per host thread at a time; each world has its own
 *    CUDA stream. Work is enqueued asynchronously; swe_world_sync(),
 *    downloads and the ledger/statistics queries wait for it.
 *  - Layout: every field is nx*nz floats, row-major [x][z] with z contiguous,
 *    index x*nz + z (math::flatten, source/include/math.h:11-14).
 *  - No entry point falls back to the CPU: without a usable CUDA device,
 *    swe_world_create fails with SWE_ERR_CUDA.
 */
#ifndef SWE_H
#define SWE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWE_OK 0
#define SWE_ERR_INVALID (-1)       /* bad argument or size                      */
#define SWE_ERR_CUDA (-2)          /* CUDA runtime error                        */
#define SWE_ERR_DEVICE (-3)        /* a kernel reported a problem in its status */
#define SWE_ERR_NO_MEMORY (-4)     /* device allocation failed                  */

/* Device status bits (swe_world_status). */
#define SWE_STATUS_NONFINITE 0x1u  /* a particle produced NaN/Inf and was retired */
#define SWE_STATUS_RANGE 0x2u      /* a fixed-point height left its safe range     */
#define SWE_STATUS_TAPE 0x4u       /* an ordered-mode rand tape ran out            */
#define SWE_STATUS_TIMEOUT 0x8u    /* a wait (barrier or cell tag) gave up; cycle aborted */

/* Simulation constants; swe_params_default() gives the reference's values.
 * Replaces the statics Wind::maxAge/boundarylayer/suspension/gravity
 * (wind.hpp:15-26), World::lrate/maxdiff/settling (world.hpp:26-32),
 * quad::mapscale (cellpool.h:184) and the per-particle prevailing wind
 * Wind::pspeed (wind.hpp:13). */
typedef struct swe_params {
  int max_age;          /* 512   */
  float boundarylayer;  /* 2.0   */
  float suspension;     /* 0.05  */
  float gravity;        /* 0.1   */
  float lrate;          /* 0.1   */
  float maxdiff;        /* 0.005 */
  float settling;       /* 1.0   */
  float mapscale;       /* 80    */
  float pspeed[3];      /* (1,0,0) */
  int frac_bits;        /* parallel mode: fixed-point fraction bits, 8..28 (24) */
  int lanes;            /* parallel mode: particles in flight at once (0) */
} swe_params;

/* Per-cell fields, in the order of quad::cell (cellpool.h:226-240). */
typedef enum swe_field {
  SWE_HEIGHT = 0,
  SWE_MASSFLOW = 1,
  SWE_MOMENTUMX = 2,
  SWE_MOMENTUMY = 3,
  SWE_MOMENTUMZ = 4,
  SWE_MASSFLOW_TRACK = 5,
  SWE_MOMENTUMX_TRACK = 6,
  SWE_MOMENTUMY_TRACK = 7,
  SWE_MOMENTUMZ_TRACK = 8
} swe_field;

/* How World::erode's particles are run.
 *  ORDERED:  particles one after another, exactly as the reference
 *            (world.hpp:47-67), with the C library rand() sequence of
 *            srand(seed) (or a caller tape) and the C library's expf: the
 *            reference's results bit for bit. One GPU thread; a parity mode.
 *  PARALLEL: the particles of a cycle fly in lock-step steps, at most
 *            `lanes` of them at a time; a lane whose particle dies takes the
 *            cycle's next particle (lanes = 0: max(1024, nx*nz/256), which
 *            keeps the terrain statistics of the sequential reference;
 *            lanes < 0: all particles at once, fastest, statistically
 *            further from the reference). In a step every particle flies
 *            against the heights as they were at the start of the step and
 *            adds its erosion/deposition to the map in fixed point; then the
 *            cascades the step owes run in a fixed conflict-free order (nine
 *            cell colours x%3, z%3). Mass is conserved exactly and the result
 *            does not depend on thread scheduling. Random numbers come from a
 *            counter-based generator keyed by (seed, cycle, particle, age). */
typedef enum swe_mode { SWE_MODE_ORDERED = 0, SWE_MODE_PARALLEL = 1 } swe_mode;

typedef struct swe_world swe_world;

/* The reference's constants (see swe_params). */
void swe_params_default(swe_params* p);

/* Allocate a world of nx*nz cells on the current CUDA device, all fields
 * zero. Replaces mappool::pool::reserve + quad::map::init node setup
 * (cellpool.h:121-164, 339-356) and srand(SEED) (SimpleWindErosion.cpp:27-34):
 * `seed` seeds both the ordered-mode rand() replica and the parallel-mode
 * generator. */
int swe_world_create(int nx, int nz, const swe_params* p, uint64_t seed, swe_world** out);
void swe_world_destroy(swe_world* w);
int swe_world_set_params(swe_world* w, const swe_params* p);
int swe_world_get_params(swe_world* w, swe_params* p);
int swe_world_size(swe_world* w, int* nx, int* nz);

/* Copy one field host -> device / device -> host (n must be nx*nz).
 * Replaces direct cell access (cell->height etc., cellpool.h:226-240,
 * SimpleWindErosion.cpp:224-230). Uploading SWE_HEIGHT resets the mass
 * ledger. */
int swe_world_upload(swe_world* w, swe_field f, const float* host, size_t n);
int swe_world_download(swe_world* w, swe_field f, float* host, size_t n);

/* An initial terrain, built on the device into SWE_HEIGHT (the other fields
 * keep their values; like an upload of SWE_HEIGHT it resets the mass ledger).
 * octaves == 0 gives the reference's own map::init terrain
 * (cellpool.h:380-428): a Gaussian bump exp(-d^2 * nx * 0.2) around
 * (nx/4, nz/2), normalised to [0, top] against min/max that include 0.
 * octaves > 0 gives fractional Brownian motion of improved gradient noise
 * (octave k at frequency base_freq * lacunarity^k with amplitude
 * persistence^k; permutation and offsets drawn from splitmix64 seeded with
 * `seed`), scaled to [0, top]. Then `npyramids` square pyramids of bedrock
 * (cx, cz, height, base in cells: height at the centre, zero at base/2) are
 * added, and `sediment` plus `sediment_jitter` times a uniform draw in
 * [-1, 1) per cell. No counterpart beyond map::init: the reference's
 * FastNoiseLite octave loop is commented out (cellpool.h:388-411). */
typedef struct swe_terrain {
  uint64_t seed;
  int octaves;
  float base_freq;
  float lacunarity;
  float persistence;
  float top;
  float sediment;
  float sediment_jitter;
  int npyramids;
  const float* pyramids; /* host array, npyramids x 4 floats */
} swe_terrain;

/* The reference's terrain: the bump (octaves 0) in [0, 0.5], nothing added. */
void swe_terrain_default(swe_terrain* t);
int swe_world_terrain(swe_world* w, const swe_terrain* t);

/* Device address of a field (nx*nz floats), for zero-copy callers. Valid until
 * swe_world_destroy; after a PARALLEL erode, SWE_HEIGHT holds the fixed-point
 * map converted back to float. */
int swe_world_device_field(swe_world* w, swe_field f, void** dev_ptr);

/* World::erode(particles_per_cycle), `cycles` times (world.hpp:36-77):
 * track reset, particle flights, EMA update of massflow/momentum. Asynchronous
 * on the world's stream. A PARALLEL call can be captured into a CUDA graph on
 * the world's stream once a first PARALLEL call with the same particle count
 * has run outside the capture (it allocates the buffers); every replay of
 * the graph is one more erode cycle (the cycle counter that keys the random
 * numbers lives on the device). */
int swe_world_erode(swe_world* w, int cycles, int particles_per_cycle, swe_mode mode);

/* The PARALLEL mode's cycle counter: the number of parallel erode cycles
 * the world has run, which keys its random numbers together with the seed.
 * A checkpoint is the nine fields (swe_world_download), the seed and this
 * counter; a world created with the same seed and parameters, given the
 * fields (swe_world_upload) and the counter, continues exactly as the
 * original would. (The reference has no checkpointing; its ORDERED-mode
 * counterpart is the C library rand() state, which a caller can replay with
 * swe_world_seed_rand plus a rand tape.) The getter waits for the stream. */
int swe_world_get_cycle(swe_world* w, uint64_t* cycle);
int swe_world_set_cycle(swe_world* w, uint64_t cycle);

/* Launch form of the PARALLEL kernel for a bounded number of particles in
 * flight: kind 0 = the default rule (one 16-CTA thread-block cluster up to
 * 4,096 lanes, else one CTA per SM), 1 = one cluster (up to 16,384 lanes),
 * 2 = a cooperative grid of `ctas` CTAs (0: one per SM; at most 4 per SM),
 * 3 = the same with 128 threads per CTA and the CTA's lanes spread over its
 * four warps (for at most 96 lanes per CTA; more take the packed grid).
 * The form changes no result, only speed; a form that cannot hold the lanes
 * falls back to the default. swe_world_tune is the autotuner: it times one
 * cycle of `particles` particles in each candidate form (default, cluster,
 * grids of one per SM, of 3/4, 1/2 and 1/4 of the SMs, and of 2, 3 and 4
 * CTAs per SM, spread grids of 1 and 2 CTAs per SM) on a scratch copy of
 * the world (its size,
 * parameters, seed and heights; the world itself is not touched), keeps the
 * fastest for the world, caches it for the process per (size, particles,
 * lanes), and reports it with its time and the default form's time (0 when
 * the form came from the cache). No counterpart in the reference, which
 * runs one particle at a time (world.hpp:47-63). */
int swe_world_set_form(swe_world* w, int kind, int ctas);
int swe_world_get_form(swe_world* w, int* kind, int* ctas);
int swe_world_tune(swe_world* w, int particles, int* kind, int* ctas, double* best_ms, double* default_ms);

/* Deadline of every wait inside a PARALLEL cycle (a grid barrier, a cell
 * tag), in nanoseconds; 0 restores the default of 2 s. A wait that runs past
 * it sets SWE_STATUS_TIMEOUT, every thread of the cycle leaves at the same
 * barrier, and the next swe_world_sync reports SWE_ERR_DEVICE; the world's
 * maps then hold a partly run cycle (upload fresh fields to go on). No
 * counterpart in the reference (its loop never waits): it exists so the
 * abort path can be exercised on a normal, terminating workload. */
int swe_world_set_wait_limit(swe_world* w, uint64_t ns);

/* An ensemble: `cycles` PARALLEL erode cycles of worlds[i] with
 * particles_per_cycle[i] particles each, for `count` independent worlds
 * (sizes, seeds, winds and parameters of their own). Each world's result is
 * the one swe_world_erode(worlds[i], cycles, particles_per_cycle[i],
 * SWE_MODE_PARALLEL) gives. Worlds whose particles in flight fit one
 * 16-CTA cluster (at most 16,384) run together in one persistent launch,
 * each cluster taking the next world from a queue; the others run on their
 * own streams. All worlds must live on one device and be distinct. Returns
 * after the persistent launch has completed (the other worlds' cycles stay
 * asynchronous on their streams); not for stream capture. Extends the reference, which erodes one
 * world (world.hpp:36-77). */
int swe_batch_erode(swe_world* const* worlds, int count, int cycles, const int* particles_per_cycle);

/* A prepared ensemble for repeated runs and CUDA-graph capture: the same
 * computation as swe_batch_erode (each world ends as swe_world_erode would
 * leave it), with the per-world launch entries written to the device once.
 * Every world's particles in flight must fit one cluster (else
 * SWE_ERR_INVALID); the worlds must outlive the batch. With tune != 0 the
 * launch shape (CTAs per cluster 4/8/16 x threads per CTA 128/256; it
 * changes no result) is chosen by timing one cycle of each feasible shape on
 * scratch copies of the worlds, and cached for the process per batch
 * signature (the sorted sides, particle counts and lanes of its worlds);
 * tune == 0 takes 16 CTAs x 256 threads. No counterpart in the reference,
 * which erodes one world (world.hpp:36-77). */
typedef struct swe_batch swe_batch;
int swe_batch_create(swe_world* const* worlds, int count, const int* particles_per_cycle, int tune, swe_batch** out);
/* `cycles` PARALLEL erode cycles of every world of the batch, enqueued on the
 * first world's stream (ordering with work on the other worlds' streams is
 * the caller's). Enqueues memsets and one kernel launch only, so it can be
 * captured into a CUDA graph on that stream; each replay runs `cycles` more
 * cycles (the worlds' cycle counters live on the device). Heights uploaded
 * after swe_batch_create are taken into fixed point by the next direct call,
 * not by replays of a graph captured before the upload. */
int swe_batch_run(swe_batch* b, int cycles);
/* The launch shape in use; after tuning, the measured cycle time (ms) of the
 * chosen shape and of the default shape (0 when not measured). */
int swe_batch_shape(swe_batch* b, int* ctas_per_cluster, int* threads_per_cta, double* tuned_ms, double* default_ms);
/* Sets the launch shape by hand (CTAs per cluster 4, 8 or 16; threads per
 * CTA a multiple of 32 up to 256); SWE_ERR_INVALID if a world's particles in
 * flight do not fit one cluster of it. */
int swe_batch_set_shape(swe_batch* b, int ctas_per_cluster, int threads_per_cta);
void swe_batch_destroy(swe_batch* b);

/* An ensemble in ORDERED mode: `cycles` erode cycles of worlds[i] with
 * particles_per_cycle[i] particles each, every world bit for bit what
 * swe_world_erode(worlds[i], cycles, particles_per_cycle[i],
 * SWE_MODE_ORDERED) gives, i.e. what the reference's World::erode
 * (world.hpp:36-77) computes from that world's rand() state or rand tape.
 * One world's particles are sequential, so each world runs on one GPU
 * thread; the ensemble's throughput comes from running many worlds at once
 * (one launch per cycle and sweep for all of them). All worlds must live on
 * one device and be distinct. Runs on the first world's stream after the
 * work queued on every world's stream, and returns after it has completed;
 * device statuses (an exhausted rand tape) are reported per world by
 * swe_world_sync. Extends the reference, which erodes one world. */
int swe_batch_erode_ordered(swe_world* const* worlds, int count, int cycles, const int* particles_per_cycle);

/* Wait for the world's queued work; returns SWE_ERR_DEVICE if a kernel set a
 * status bit since the last call (bits in *status if non-NULL, then cleared). */
int swe_world_sync(swe_world* w);
int swe_world_status(swe_world* w, uint32_t* status);

/* Ordered mode random source. swe_world_seed_rand reseeds the rand() replica
 * (srand, SimpleWindErosion.cpp:29/33). swe_world_set_rand_tape makes ordered
 * erodes consume the given raw rand() values in call order instead (4 per
 * spawn, world.hpp:52-54; 3 per successful step, wind.hpp:83); n = 0 returns
 * to the replica. */
int swe_world_seed_rand(swe_world* w, uint32_t seed);
int swe_world_set_rand_tape(swe_world* w, const int32_t* tape, size_t n);

/* Mass ledger of the parallel mode in fixed point (units of 2^-frac_bits):
 * map_q = sum of heights, inflight_q = sediment carried by particles still
 * flying (0 between erode calls), exported_q = sediment carried off the map
 * or dropped at max_age since the last height upload. map_q + inflight_q +
 * exported_q stays constant. */
int swe_world_mass_ledger(swe_world* w, int64_t* map_q, int64_t* inflight_q, int64_t* exported_q);

/* Counters of the last swe_world_erode call: successful fly steps, spawned
 * particles, cascade transfers. */
int swe_world_stats(swe_world* w, int64_t* particle_steps, int64_t* particles, int64_t* transfers);

/* Frozen-map trajectories (Wind::fly, wind.hpp:28-117, with the map left
 * unchanged). Particle p spawns at (spawn_xz[2p], spawn_xz[2p+1]); its step s
 * draws turbulence from turb_tape[(p*steps+s)*3 + 0..2] (raw rand() values in
 * call order). out_state gets 9 floats per (p, s): alive, age, pos.xyz,
 * speed.xyz, sediment. */
int swe_trace_particles(swe_world* w, const float* spawn_xz, int n, int steps,
                        const int32_t* turb_tape, float* out_state);

/* One particle flown on the live map for up to `steps` Wind::fly calls
 * (ordered semantics, writes happen). turb_tape: 3 raw rand() values per
 * step, or NULL to draw from the rand() replica. out_state as above (may be
 * NULL). *ok_steps = successful fly calls. */
int swe_world_fly(swe_world* w, float x, float z, int steps, const int32_t* turb_tape,
                  float* out_state, int* ok_steps);

/* World::cascade at one cell (world.hpp:79-153), on the float height map. */
int swe_world_cascade_at(swe_world* w, int x, int z);

/* The surface vertices updatenode writes for rendering after each erode call
 * (cellpool.h:302-333, SimpleWindErosion.cpp:219-221): per cell 12 floats,
 * the position P = (x, mapscale*height, z), the normal (quad::_normal), and
 * the edges T-P and B-P to the +x and +z neighbours (heights off the map
 * read 0); n = 12*nx*nz floats in cell order written to host_out. A
 * headless buffer in place of the reference's vertex pool. */
int swe_world_vertices(swe_world* w, float* host_out, size_t n);

/* The wind map the reference's app loop builds after each erode call
 * (SimpleWindErosion.cpp:224-230): per cell the RGBA texel
 * (0.5(1+erf(2 momentumx)), 0.5(1+erf(2 momentumy)), 0.5(1+erf(2 momentumz)), 1),
 * 4*nx*nz floats in cell order written to host_rgba (n = 4*nx*nz). */
int swe_world_windmap(swe_world* w, float* host_rgba, size_t n);

/* Surface normal of every cell, quad::_normal (cellpool.h:200-223) as
 * map::normal calls it (cellpool.h:478-480): 3*nx*nz floats (x,y,z per cell)
 * written to host_out. */
int swe_world_normals(swe_world* w, float* host_out, size_t n);

/* The CUDA stream (a cudaStream_t) the world enqueues its work on, and a
 * way to replace it with the caller's stream (NULL: back to a private
 * stream). The world does not destroy a caller's stream. */
int swe_world_get_stream(swe_world* w, void** stream);
int swe_world_set_stream(swe_world* w, void* stream);

/* Time the parallel mode spent in its fly phases and in its cascade phases
 * (ms, the device's global timer read by one thread at the phase barriers),
 * summed over the cycles of the last swe_world_erode call. No reference
 * counterpart (the reference has no timing). */
int swe_world_kernel_times(swe_world* w, double* fly_ms, double* cascade_ms);

/* The same clock per phase of the parallel cycle kernels, ms summed over the
 * last swe_world_erode call, in the order: spawn, fly, (unused), colour 0..8,
 * ema (n <= 13 values written). The all-at-once kernel fills every slot. The
 * bounded-lanes kernel (the default) has no colour phases; its slots hold:
 * fly = flights, their tag waits and the step's barrier; colour 0 = refills,
 * absorbs and cascades; and parts of those two: spawn = the flights' tag
 * waits, (unused) = the barrier, colour 1 = refills and absorbs (its map
 * sweeps and EMA are not timed). */
int swe_world_phase_times(swe_world* w, double* ms, int n);

/* Cascade work of the last parallel swe_world_erode call: World::cascade
 * evaluations, cell-steps that owed cascades, and the most cascades one cell
 * ran in one step. */
int swe_world_cascade_stats(swe_world* w, int64_t* cascades, int64_t* cells, int* max_iters);

/* The exponential the exact-semantics kernels use (the reference's
 * std::exp(float), wind.hpp:50, i.e. this machine's C library expf,
 * reproduced on the device) evaluated for the n float bit patterns
 * first_bits, first_bits+1, ...; for checking it against the C library. */
int swe_world_expf_bits(swe_world* w, uint32_t first_bits, size_t n, float* host_y);

/* Parallel erosion that allocates no device memory. No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc, such as a
 * frame loop inside a render or game engine that owns the GPU's memory pool
 * (the reference's own app erodes once per rendered frame), or code running
 * while another framework's allocator owns the device memory.
 *
 * `fields` are the caller's nine device arrays of nx*nz floats in swe_field
 * order (inputs and outputs, as a world's fields). The call runs `cycles`
 * parallel erode cycles of `particles_per_cycle` particles (same results as a
 * world whose random-number cycle counter is `first_cycle`), enqueued on
 * `stream` (NULL: the default stream). The scratch it needs lives in one
 * static device array, about 17.1 MiB on every GPU that loads the library,
 * held until the process exits; its limits are SWE_NOALLOC_MAX_CELLS cells
 * and SWE_NOALLOC_MAX_PARTICLES particles per cycle, and larger requests fail
 * with SWE_ERR_INVALID. Particles in flight stay in the kernel's shared
 * memory (at most SMs x 1,024 of them; more are refused the same way). The first call on a device looks up that array's
 * device address (set-up, once per device): make that first call before any
 * stream capture. All calls share the array, so calls that overlap on the GPU
 * race; serialise them (one stream, or synchronise between them). If
 * `status` is non-NULL the call waits for the stream and reports the device
 * status bits (SWE_ERR_DEVICE if any are set). */
#define SWE_NOALLOC_MAX_CELLS 262144
#define SWE_NOALLOC_MAX_PARTICLES 65536
int swe_erode_parallel_noalloc(float* const* fields, int nx, int nz, const swe_params* p, uint64_t seed,
                               uint64_t first_cycle, int cycles, int particles_per_cycle, void* stream,
                               uint32_t* status);

/* ---- Learned surrogate: building blocks of a BF16 U-Net ----
 * No counterpart in the reference (an extension: a network that predicts
 * the terrain after a number of erode cycles, trained on pairs the erosion
 * path produces, with that path as its fallback and judge). Tensors are
 * device arrays in NHWC order (channels innermost); "bf16" tensors hold
 * bfloat16 values (uint16 storage) and must be 16-byte aligned (the
 * convolution's output: 4-byte); arithmetic accumulates in fp32. Every call is enqueued on `stream` (NULL: the default
 * stream) and returns once enqueued.
 *
 * y[n,i,j,co] = bias[co] + sum over the 3x3 taps (zero padding) and ci of
 * x[n,i+di,j+dj,ci] w[co,di+1,dj+1,ci]; x bf16 [n,h,w,cin], w bf16
 * [cout,3,3,cin], bias fp32 [cout] or NULL, y bf16 [n,h,w,cout]; cin a
 * multiple of 16, cout of 8. Runs on the tensor cores (implicit GEMM). */
int swe_nn_conv3x3(const void* x, const void* w, const float* bias, void* y, int n, int h, int wd, int cin, int cout,
                   void* stream);
/* The same convolution on the Blackwell tensor cores (tcgen05.mma, fp32
 * accumulators in tensor memory, TMA-fed operand tiles; a persistent kernel
 * of up to three CTAs per SM, each a copy/MMA pipeline of up to six
 * mbarrier stages, the epilogue of one pair of 128-pixel tiles under the
 * MMAs of the next). Weights come packed by swe_nn_conv3x3_tc_pack: flip == 0 packs
 * w bf16 [cout,3,3,cin] for the forward convolution (x has cin channels, y
 * cout); flip != 0 packs the flipped, transposed weights whose convolution
 * of dy (cout channels) is the input gradient (cin channels), i.e. this call
 * with cin and cout swapped. `act` (or NULL) also receives GELU(y), fused
 * into the epilogue. cin and cout multiples of 16, cout <= 256; with TW the
 * largest power of two up to 128 dividing the map width, TW >= 8 and the
 * height a multiple of 128 / TW (a 128-pixel tile is 128 / TW rows of TW
 * pixels); tensors 16-byte aligned. packed: 9*cin*cout bf16. */
int swe_nn_conv3x3_tc_pack(const void* w, void* wp, int cin, int cout, int flip, void* stream);
int swe_nn_conv3x3_tc(const void* x, const void* wp, const float* bias, void* y, void* act, int n, int h, int wd,
                      int cin, int cout, void* stream);
/* Weight and bias gradients of swe_nn_conv3x3 on the tensor cores, ADDED to
 * dw (fp32 [cout,3,3,cin]) and db (fp32 [cout], or NULL): per tap a GEMM
 * with M = output channels, N = input channels, K = pixels (split over
 * CTAs, partial sums added with fp32 atomics); the bias gradient in the same
 * kernel, dy against a block of ones. cin and cout multiples of 16
 * up to 128; map shape as for swe_nn_conv3x3_tc; x and dy 16-byte aligned. */
int swe_nn_conv3x3_wgrad_tc(const void* x, const void* dy, float* dw, float* db, int n, int h, int wd, int cin,
                            int cout, void* stream);
/* SWE_ERR_DEVICE (code in *status) if a tensor-core kernel gave up on a wait
 * since the last call (each wait has a 2 s deadline); clears the code. Call
 * after synchronising the streams the kernels ran on. */
int swe_nn_status(uint32_t* status);
/* wf[ci,2-di,2-dj,co] = w[co,di,dj,ci]: the weights whose convolution of dy
 * is the input gradient of swe_nn_conv3x3. */
int swe_nn_conv3x3_flip(const void* w, void* wf, int cin, int cout, void* stream);
/* Weight and bias gradients of swe_nn_conv3x3, ADDED to dw (fp32
 * [cout,3,3,cin]) and db (fp32 [cout], or NULL) from its input x and the
 * output gradient dy (bf16 [n,h,w,cout]); cout <= 256, x and dy 16-byte
 * aligned. */
int swe_nn_conv3x3_wgrad(const void* x, const void* dy, float* dw, float* db, int n, int h, int wd, int cin, int cout,
                         void* stream);
/* act = GELU(pre) = pre (1 + erf(pre / sqrt 2)) / 2, and dpre = dact GELU'(pre).
 * For these and the pooling, upsampling and add calls: counts and channel
 * numbers are multiples of 8 and tensors 16-byte aligned. */
int swe_nn_gelu(const void* pre, void* act, int64_t count, void* stream);
int swe_nn_gelu_bwd(const void* pre, const void* dact, void* dpre, int64_t count, void* stream);
/* 2x2 average pooling of x [n,h,w,c] (h, w even) into y [n,h/2,w/2,c]; with
 * backward != 0, x is the gradient [n,h/2,w/2,c] and y the input gradient
 * [n,h,w,c]. */
int swe_nn_pool2(const void* x, void* y, int n, int h, int wd, int c, int backward, void* stream);
/* Nearest 2x upsampling of x [n,h,w,c] into y [n,2h,2w,c]; with backward !=
 * 0, x is the gradient [n,2h,2w,c] and y the input gradient [n,h,w,c]. */
int swe_nn_up2(const void* x, void* y, int n, int h, int wd, int c, int backward, void* stream);
/* out = a + b (bf16, elementwise). */
int swe_nn_add(const void* a, const void* b, void* out, int64_t count, void* stream);
/* The network input, 16 bf16 channels per cell: (height - 0.25) * 4, the
 * wind direction's x and z components (wind_xz: 2 floats per map), zeros.
 * height fp32 [n,h,w]. */
int swe_nn_pack_input(const float* height, const float* wind_xz, void* x, int n, int h, int wd, void* stream);
/* The same with every map's heights moved by a constant so that its mean is
 * `ref`: channel 0 = ((height - mean) + (ref - 0.25)) * 4, mean = the map's
 * mean height, also written to means (device, n floats). The erosion rules
 * see heights only through differences (slopes, normals, the particle's
 * height above the cell, cascades), so the change over a jump does not
 * depend on such a constant; the network then sees every terrain at the
 * height level it was trained on. */
int swe_nn_pack_input_centered(const float* height, const float* wind_xz, float* means, void* x, int n, int h, int wd,
                               float ref, void* stream);
/* Squared error of channel 0 of pred (bf16 [pixels, c]) against target *
 * target_scale (target fp32 [pixels]): the sum of squares is ADDED to *loss
 * (device fp32) and dpred = 2 (pred - target target_scale) grad_scale on
 * channel 0, 0 on the others. */
int swe_nn_mse(const void* pred, const float* target, float target_scale, void* dpred, float* loss, int64_t pixels,
               int c, float grad_scale, void* stream);
/* out[p] = channel 0 of pred (bf16 [pixels, c]) times out_scale, as fp32. */
int swe_nn_channel0(const void* pred, float* out, int64_t pixels, int c, float out_scale, void* stream);
/* One Adam step (step = 1, 2, ...) on fp32 weights w with gradient grad and
 * moments m, v; w_bf16 (or NULL) receives the updated weights as bf16. */
int swe_nn_adam(float* w, const float* grad, float* m, float* v, void* w_bf16, int64_t count, float lr, float beta1,
                float beta2, float eps, int step, void* stream);
/* b = bf16(a). */
int swe_nn_to_bf16(const float* a, void* b, int64_t count, void* stream);

/* Message of the calling thread's last error ("" if none). */
const char* swe_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* SWE_H */
