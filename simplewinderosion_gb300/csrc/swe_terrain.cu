// Initial terrains on the device.
//
// The reference builds its map in map::init (source/cellpool.h:336-428): a
// Gaussian bump exp(-d^2 * tilesize * 0.2) around (1/4, 1/2) of the map,
// normalised to [0, 0.5] against min/max that start at 0 (its FastNoiseLite
// fBm loop is commented out, :388-411). The workloads here also need seeded
// fBm terrains with pyramids of bedrock and a sediment layer; building them
// on the host takes seconds per 1024^2 map and minutes at 4096^2, so they
// are built here, two passes over the map:
//   eval    bedrock value per cell (the bump, or fBm of improved gradient
//           noise: K. Perlin, "Improving Noise", SIGGRAPH 2002, quintic fade,
//           gradients hashed through a seeded permutation), and its min/max;
//   finish  scale to [0, top], add pyramids, sediment and per-cell jitter.
// The noise is evaluated in double precision; the permutation, offsets and
// jitter come from splitmix64 (S. Vigna), so a host restatement of the same
// steps reproduces the map to rounding.
#include <cuda_runtime.h>

#include <cstdint>

#include "swe_device.cuh"
#include "swe_kernels.h"

namespace swe {
namespace {

__host__ __device__ inline uint64_t splitmix64_next(uint64_t& s) {
  s += 0x9E3779B97F4A7C15ull;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Uniform double in [0, 1) from the top 53 bits.
__host__ __device__ inline double unit53(uint64_t v) { return (double)(v >> 11) * (1.0 / 9007199254740992.0); }

__device__ inline double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }

__device__ inline double grad2(int h, double dx, double dy) {
  // gradients (1,1) (-1,1) (1,-1) (-1,-1) (1,0) (-1,0) (0,1) (0,-1)
  switch (h & 7) {
    case 0: return dx + dy;
    case 1: return -dx + dy;
    case 2: return dx - dy;
    case 3: return -dx - dy;
    case 4: return dx;
    case 5: return -dx;
    case 6: return dy;
    default: return -dy;
  }
}

__device__ inline double perlin2(double x, double y, const int* perm) {
  const double fx = floor(x), fy = floor(y);
  const int xi = (int)((long long)fx & 255), yi = (int)((long long)fy & 255);
  const double xf = x - fx, yf = y - fy;
  const double u = fade(xf), v = fade(yf);
  const int aa = perm[perm[xi] + yi], ab = perm[perm[xi] + yi + 1];
  const int ba = perm[perm[xi + 1] + yi], bb = perm[perm[xi + 1] + yi + 1];
  const double x1 = grad2(aa, xf, yf) * (1.0 - u) + grad2(ba, xf - 1.0, yf) * u;
  const double x2 = grad2(ab, xf, yf - 1.0) * (1.0 - u) + grad2(bb, xf - 1.0, yf - 1.0) * u;
  return x1 * (1.0 - v) + x2 * v;
}

// Order-preserving map of doubles to unsigned 64-bit keys (for atomic min/max).
__device__ inline unsigned long long dkey(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ inline double dkey_inv(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double((long long)b);
}

struct TerrainArgs {
  int nx, nz;
  int octaves;  // 0: the reference's bump
  double base_freq, lacunarity, persistence, offx, offz;
  int perm[512];
};

__global__ void k_terrain_eval(TerrainArgs a, double* __restrict__ val, unsigned long long* minmax) {
  __shared__ int perm[512];
  for (int k = threadIdx.x; k < 512; k += blockDim.x) perm[k] = a.perm[k];
  __syncthreads();
  const long n = (long)a.nx * a.nz;
  double lo = 1e300, hi = -1e300;
  if (a.octaves == 0) {
    // map::init (cellpool.h:380-385) in float, the exponential in double:
    // p = pos/tileres, c = (tileres/ivec2(4,2))/tileres, d = length(p - c),
    // height = exp(-d*d*tilesize*0.2); min and max start at 0 (:416-421).
    lo = 0.0;
    hi = 0.0;
  }
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i / a.nz), z = (int)(i - (long)x * a.nz);
    double v;
    if (a.octaves == 0) {
      const float px = (float)x / (float)a.nx, pz = (float)z / (float)a.nz;
      const float cx = (float)(a.nx / 4) / (float)a.nx, cz = (float)(a.nz / 2) / (float)a.nz;
      const float dx = px - cx, dz = pz - cz;
      const float d = sqrtf(dx * dx + dz * dz);
      const float t = -d * d * (float)a.nx;
      v = (double)(float)exp((double)t * 0.2);
    } else {
      v = 0.0;
      double amp = 1.0, f = a.base_freq;
      for (int o = 0; o < a.octaves; o++) {
        v += amp * perlin2((double)x * f + a.offx, (double)z * f + a.offz, perm);
        amp *= a.persistence;
        f *= a.lacunarity;
      }
    }
    val[i] = v;
    lo = fmin(lo, v);
    hi = fmax(hi, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(minmax, dkey(lo));
    atomicMax(minmax + 1, dkey(hi));
  }
}

struct FinishArgs {
  int nx, nz;
  int bump;
  double top, sediment, jitter;
  uint64_t jitter_seed;
  int npyr;
  const float* pyr;  // npyr x (cx, cz, height, base)
};

__global__ void k_terrain_finish(FinishArgs a, const double* __restrict__ val, const unsigned long long* minmax,
                                 float* __restrict__ H) {
  const long n = (long)a.nx * a.nz;
  const double lo = dkey_inv(minmax[0]), hi = dkey_inv(minmax[1]);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i / a.nz), z = (int)(i - (long)x * a.nz);
    double h;
    if (a.bump) {
      // cell.height = 0.5*((cell.height - min)/(max - min)) (cellpool.h:423-426):
      // the difference and quotient in float, the 0.5 in double
      const float fl = (float)lo, fh = (float)hi, fv = (float)val[i];
      h = a.top * (double)((fv - fl) / (fh - fl));
    } else {
      h = hi > lo ? (val[i] - lo) / (hi - lo) * a.top : 0.0;
    }
    for (int k = 0; k < a.npyr; k++) {
      const double cx = a.pyr[4 * k], cz = a.pyr[4 * k + 1], ph = a.pyr[4 * k + 2], base = a.pyr[4 * k + 3];
      const double d = fmax(fabs((double)x - cx), fabs((double)z - cz)) / (base / 2.0);
      h += ph * fmax(1.0 - d, 0.0);
    }
    if (a.sediment != 0.0 || a.jitter != 0.0) {
      uint64_t s = a.jitter_seed + (uint64_t)i * 0x9E3779B97F4A7C15ull;
      h += a.sediment + a.jitter * (2.0 * unit53(splitmix64_next(s)) - 1.0);
    }
    H[i] = (float)h;
  }
}

}  // namespace

cudaError_t launch_terrain(float* height, int nx, int nz, const TerrainSpec& t, cudaStream_t s) {
  const long n = (long)nx * nz;
  TerrainArgs a{};
  a.nx = nx;
  a.nz = nz;
  a.octaves = t.octaves;
  a.base_freq = t.base_freq;
  a.lacunarity = t.lacunarity;
  a.persistence = t.persistence;
  // permutation (Fisher-Yates) and offsets from splitmix64 seeded with t.seed
  uint64_t st = t.seed;
  int p[256];
  for (int k = 0; k < 256; k++) p[k] = k;
  for (int k = 255; k > 0; k--) {
    const int j = (int)(splitmix64_next(st) % (uint64_t)(k + 1));
    const int tmp = p[k];
    p[k] = p[j];
    p[j] = tmp;
  }
  for (int k = 0; k < 512; k++) a.perm[k] = p[k & 255];
  a.offx = 256.0 * unit53(splitmix64_next(st));
  a.offz = 256.0 * unit53(splitmix64_next(st));

  FinishArgs f{};
  f.nx = nx;
  f.nz = nz;
  f.bump = t.octaves == 0;
  f.top = t.top;
  f.sediment = t.sediment;
  f.jitter = t.sediment_jitter;
  f.jitter_seed = splitmix64_next(st);
  f.npyr = t.npyramids;

  void* scratch = nullptr;
  const size_t pyr_bytes = sizeof(float) * 4 * (size_t)t.npyramids;
  const size_t bytes = 256 + sizeof(double) * (size_t)n + pyr_bytes;
  cudaError_t e = cudaMallocAsync(&scratch, bytes, s);
  if (e != cudaSuccess) return e;
  unsigned long long* minmax = static_cast<unsigned long long*>(scratch);
  double* val = reinterpret_cast<double*>(static_cast<char*>(scratch) + 256);
  float* pyr = reinterpret_cast<float*>(static_cast<char*>(scratch) + 256 + sizeof(double) * (size_t)n);
  const unsigned long long init[2] = {~0ull, 0ull};
  e = cudaMemcpyAsync(minmax, init, sizeof(init), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && pyr_bytes) e = cudaMemcpyAsync(pyr, t.pyramids, pyr_bytes, cudaMemcpyHostToDevice, s);
  f.pyr = pyr;
  if (e == cudaSuccess) {
    long g = (n + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    if (g < 1) g = 1;
    k_terrain_eval<<<(int)g, 256, 0, s>>>(a, val, minmax);
    k_terrain_finish<<<(int)g, 256, 0, s>>>(f, val, minmax, height);
    e = cudaGetLastError();
  }
  // the host copies above read `init` and the pyramids before this returns
  const cudaError_t es = cudaStreamSynchronize(s);
  cudaFreeAsync(scratch, s);
  return e != cudaSuccess ? e : es;
}

}  // namespace swe
