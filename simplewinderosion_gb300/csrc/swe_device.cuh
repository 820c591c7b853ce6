// Device-side arithmetic shared by the erosion kernels.
//
// Every translation unit of the library is compiled with -fmad=false: each
// float multiply and add is rounded on its own, as in the reference built
// with g++ -O2 on x86-64 (no contraction), and fused multiply-adds appear only
// where fmaf() is written out. sqrtf and '/' are the IEEE correctly rounded
// forms (no fast-math), so the vector helpers below reproduce the glm
// semantics the reference relies on:
//   dot = (x*x' + y*y') + z*z',  normalize(v) = v * (1/sqrt(dot(v,v))),
//   cross = (a.y b.z - b.y a.z, a.z b.x - b.z a.x, a.x b.y - b.x a.y),
//   mix(x,y,a) = x*(1-a) + y*a.
#pragma once

#include <cstdint>

#include "swe_types.h"

namespace swe {

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 smul(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ V3 muls(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ V3 subs(V3 a, float s) { return v3(a.x - s, a.y - s, a.z - s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float length(V3 v) { return sqrtf(dot(v, v)); }
__device__ __forceinline__ V3 normalize(V3 v) { return muls(v, 1.0f / sqrtf(dot(v, v))); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ V3 mix(V3 x, V3 y, float a) { return add(muls(x, 1.0f - a), muls(y, a)); }

// Neighbour offsets in World::cascade's order (world.hpp:83-92).
__device__ __constant__ static const int kNbDx[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
__device__ __constant__ static const int kNbDz[8] = {-1, 0, 1, -1, 1, -1, 0, 1};

// Surface normal of quad::_normal (cellpool.h:200-223). h(x,z) returns the
// height of an in-bounds cell; the oob gates are the reference's diagonal
// checks, so h is only called on in-bounds cells.
template <class H>
__device__ __forceinline__ V3 surface_normal(int x, int z, int nx, int nz, float mapscale, H h) {
  auto oob = [&](int a, int b) { return a < 0 || b < 0 || a >= nx || b >= nz; };
  V3 n = v3(0.0f, 0.0f, 0.0f);
  const V3 s = v3(1.0f, mapscale, 1.0f);
  const float hp = h(x, z);
  if (!oob(x + 1, z + 1))
    n = add(n, cross(mulv(s, v3(0.0f, h(x, z + 1) - hp, 1.0f)), mulv(s, v3(1.0f, h(x + 1, z) - hp, 0.0f))));
  if (!oob(x - 1, z - 1))
    n = add(n, cross(mulv(s, v3(0.0f, h(x, z - 1) - hp, -1.0f)), mulv(s, v3(-1.0f, h(x - 1, z) - hp, 0.0f))));
  if (!oob(x + 1, z - 1))
    n = add(n, cross(mulv(s, v3(1.0f, h(x + 1, z) - hp, 0.0f)), mulv(s, v3(0.0f, h(x, z - 1) - hp, -1.0f))));
  if (!oob(x - 1, z + 1))
    n = add(n, cross(mulv(s, v3(-1.0f, h(x - 1, z) - hp, 0.0f)), mulv(s, v3(0.0f, h(x, z + 1) - hp, 1.0f))));
  if (length(n) > 0.0f) n = normalize(n);
  return n;
}

// The reference's std::exp(float) (source/wind.hpp:50), i.e. the C library
// expf, bit for bit: the double exponential rounded once to float is the
// correctly rounded value; only when it lies within 1% of an ulp of a
// rounding midpoint can the C library (about 0.502 ulp accurate) differ, and
// the build-time list of such arguments (c.expf_x, from the C library
// itself) gives the one-ulp correction.
__device__ __forceinline__ float exp_libm(float x, const Consts& c) {
  const double e = exp((double)x);
  float r = (float)e;
  const float lo = __double2float_rd(e), hi = __double2float_ru(e);
  if (lo != hi) {
    const double mid = 0.5 * ((double)lo + (double)hi);
    if (fabs(e - mid) < 0.01 * ((double)hi - (double)lo)) {
      const uint32_t key = __float_as_uint(x);
      int a = 0, b = c.expf_n;
      while (a < b) {
        const int m = (a + b) >> 1;
        if (c.expf_x[m] < key) a = m + 1; else b = m;
      }
      if (a < c.expf_n && c.expf_x[a] == key)
        r = nextafterf(r, c.expf_d[a] > 0 ? __int_as_float(0x7f800000) : __int_as_float(0xff800000));
    }
  }
  return r;
}

// Own single-precision exp for the parallel mode: Cody-Waite reduction
// x = k ln2 + r, degree-7 Taylor polynomial of e^r (|r| <= ln2/2) in Horner
// form with fused multiply-adds, 2^k applied through the exponent field.
// Results below e^-86 flush to zero. Bit-identical to the CPU model because
// it uses only correctly rounded IEEE operations.
__device__ __forceinline__ float expf_poly(float x) {
  if (!(x == x)) return x;
  if (x < -86.0f) return 0.0f;
  if (x > 88.0f) return __int_as_float(0x7f800000);
  const float k = rintf(x * 1.44269504f);
  float r = fmaf(k, -0.693145752f, x);
  r = fmaf(k, -1.42860677e-6f, r);
  float p = 1.98412698e-4f;
  p = fmaf(p, r, 1.38888889e-3f);
  p = fmaf(p, r, 8.33333333e-3f);
  p = fmaf(p, r, 4.16666667e-2f);
  p = fmaf(p, r, 1.66666667e-1f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  const int ki = (int)k;
  return p * __int_as_float((ki + 127) << 23);
}

// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): ten rounds with the paper's multipliers and Weyl
// key increments.
__device__ __forceinline__ uint4 philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                            uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int round = 0; round < 10; round++) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return make_uint4(c0, c1, c2, c3);
}

// Float to fixed point, round to nearest even, saturating (NaN -> 0).
__device__ __forceinline__ int32_t to_fixed(float v) { return __float2int_rn(v); }
__device__ __forceinline__ long long to_fixed64(float v) { return __float2ll_rn(v); }

}  // namespace swe
