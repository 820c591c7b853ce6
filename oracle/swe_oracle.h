/* TEST INFRASTRUCTURE — CPU oracle for the SimpleWindErosion hot path.
 *
 * A plain C++ restatement of the reference's World::erode / Wind::fly /
 * World::cascade / quad::_normal (source/world.hpp:36-153,
 * source/wind.hpp:28-117, source/cellpool.h:200-223) over SoA float maps,
 * plus a CPU model of the library's parallel fixed-point mode. Only tests,
 * the smoke check and the bench's CPU legs load it; the product library never
 * links or calls it.
 *
 * Bit-for-bit equal to the reference compiled from its own headers
 * (oracle/ref_harness.cpp) when rng = SO_RNG_LIBC or SO_RNG_GLIBC and
 * exp_kind = SO_EXP_LIBM; checked by tests/test_oracle_vs_reference.py.
 */
#ifndef SWE_ORACLE_H
#define SWE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct so_params {
  int max_age;          /* Wind::maxAge        wind.hpp:23 */
  float boundarylayer;  /* Wind::boundarylayer wind.hpp:24 */
  float suspension;     /* Wind::suspension    wind.hpp:25 */
  float gravity;        /* Wind::gravity       wind.hpp:26 */
  float lrate;          /* World::lrate        world.hpp:30 */
  float maxdiff;        /* World::maxdiff      world.hpp:31 */
  float settling;       /* World::settling     world.hpp:32 */
  float mapscale;       /* quad::mapscale      cellpool.h:184 */
  float pspeed[3];      /* Wind::pspeed        wind.hpp:13 */
  int frac_bits;        /* parallel model: fixed-point fraction bits */
  int lanes;            /* parallel model: particles in flight (0 auto, <0 all) */
} so_params;

enum { SO_RNG_LIBC = 0, SO_RNG_GLIBC = 1, SO_RNG_TAPE = 2 };
enum { SO_EXP_LIBM = 0, SO_EXP_CR = 1 };

typedef struct so_world so_world;

void so_params_default(so_params* p);
so_world* so_create(int nx, int nz, const so_params* p);
void so_destroy(so_world* w);
void so_set_field(so_world* w, int field, const float* src);
void so_get_field(so_world* w, int field, float* dst);
void so_set_params(so_world* w, const so_params* p);

/* rng: SO_RNG_LIBC uses the process-wide rand() (call srand first);
 * SO_RNG_GLIBC uses the world's own replica of that generator. */
void so_set_rng(so_world* w, int rng, uint32_t seed);
void so_set_exp(so_world* w, int exp_kind);
void so_set_tape(so_world* w, const int32_t* tape, long n);
long so_tape_pos(so_world* w);

void so_erode(so_world* w, int particles, int cycles);
void so_normal(so_world* w, int x, int z, float* out3);
void so_cascade(so_world* w, int x, int z);
int so_trace(so_world* w, int n, const float* spawn_xz, int steps, const int32_t* tape, float* out);
int so_fly_live(so_world* w, float x, float z, int steps, const int32_t* tape, float* out);

/* Counters of the last so_erode call: particle-steps (successful fly calls),
 * spawned particles, and cascade transfers. */
void so_stats(so_world* w, int64_t* steps, int64_t* particles, int64_t* transfers);

/* The C library rand() sequence after srand(seed), from the replica. */
void so_glibc_rand_sequence(uint32_t seed, int n, int32_t* out);

/* --- CPU model of the parallel fixed-point mode (bitwise model of the GPU
 *     kernels: same float operation order, same counter-based RNG). --- */
void so_par_erode(so_world* w, int particles, int cycles, uint64_t seed, uint64_t* cycle_counter);
// Which particles of a cycle fly together in so_par_erode (default 0): 0 the
// library's rule (freed lanes take the cycle's next ids); 1 lane k takes ids
// k, k + L, k + 2L, ...; 2 a fixed schedule, particle j spawning at step
// floor(400 j / L) (L in flight on average). Modes 1 and 2 are explorations
// for a parallel mode without a global step barrier; the library runs mode 0.
void so_par_set_spawn_mode(so_world* w, int mode);
// The last so_par_erode call's largest one-step move of a particle along x or
// z, in cells (the reach a cell's visitors can come from).
float so_par_max_move(so_world* w);
/* Particles in flight at once: lanes > 0 as given, 0 -> max(1024, cells/256),
 * < 0 -> all particles of the cycle; never more than the cycle's particles. */
int so_par_lanes(int lanes, int nx, int nz, int particles);
void so_par_get_heights_q(so_world* w, int32_t* dst);
void so_par_ledger(so_world* w, int64_t* map_q, int64_t* exported_q);
void so_philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                   uint32_t* out4);
float so_expf_poly(float x);
/* The C library expf over n consecutive float bit patterns. */
void so_expf_libm_bits(uint32_t first, long n, float* out);

#ifdef __cplusplus
}
#endif
#endif
