// Plain structs shared by the host world object and the kernels.
#pragma once

#include <cstdint>

namespace swe {

// Constants of one world, passed to kernels by value (mirrors swe_params).
struct Consts {
  int nx, nz;
  int max_age;
  float boundarylayer, suspension, gravity, lrate, maxdiff, settling, mapscale;
  float px, py, pz;  // prevailing wind (Wind::pspeed)
  int frac_bits;
  float scale;      // 2^frac_bits
  float inv_scale;  // 2^-frac_bits
  // Arguments where the C library expf is not the correctly rounded value
  // (sorted bit patterns) and the direction of its one-ulp difference.
  const uint32_t* expf_x;
  const int8_t* expf_d;
  int expf_n;
  // Parallel mode: how long one wait (a grid barrier or a cell tag) may
  // spin before the cycle is aborted with SWE_STATUS_TIMEOUT; 0 = 2 s.
  unsigned long long wait_ns;
};

// State of the C library rand() replica: the last 34 elements of the
// additive feedback recurrence r[i] = r[i-31] + r[i-3] (mod 2^32), element i
// in slot i % 34, and the slot of the next element to produce.
struct GlibcRandState {
  uint32_t r[34];
  int head;
  int pad;
};

// Device-side counters of one world (one allocation, zeroed per erode call).
struct Counters {
  unsigned long long particle_steps;
  unsigned long long particles;
  unsigned long long transfers;
  long long exported_q;      // cumulative since the last height upload
  int live[2];               // parallel mode: survivors appended per step parity
  int refill[2];             // parallel mode: particles spawned into freed lanes, per step parity
  int next_id[2];            // parallel mode: next particle id to spawn, per step parity
  unsigned int status;       // SWE_STATUS_* bits
  unsigned int pad;
  long long tape_pos;        // ordered mode tape cursor
  unsigned long long cycle;  // parallel mode: cycles completed (RNG counter)
  unsigned long long fly_ns;      // parallel mode: time in fly phases (block 0's clock)
  unsigned long long cascade_ns;  // parallel mode: time in apply + colour phases
  // parallel mode, per phase (block 0's clock, barrier included):
  // spawn, fly, (unused), colour 0..8, ema
  unsigned long long phase_ns[13];
  unsigned long long cascades;       // parallel mode: World::cascade evaluations
  unsigned long long cascade_cells;  // parallel mode: cell-steps with owed cascades
  unsigned int max_cascade_iters;    // parallel mode: most cascades of one cell in one step
  unsigned int pad2;
};

// State of the grid-wide barriers of the persistent parallel kernels (one
// arrival atomic per block: every block adds 1 but block 0, which adds
// 2^31 - (blocks - 1), so the top bit of `flip` flips when the last block
// arrives), and three counters (one per step mod 3) that the bounded-lanes
// kernel's barrier sums a per-block count into on the way.
struct GridBarrier {
  unsigned int flip;
  unsigned int abort;  // set by a thread that gave up waiting
  unsigned int pad[30];
  unsigned int sums[3 * 32];  // one 128-byte line each
};

// Particle state of the parallel mode, structure of arrays.
struct ParticleSoA {
  int* id;
  int* age;
  float* px;
  float* py;
  float* pz;
  float* vx;
  float* vy;
  float* vz;
  int* sed_q;
};

}  // namespace swe
