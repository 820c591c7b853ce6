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

// ---- float-float arithmetic: a value is the unevaluated sum hi + lo ----
// TwoSum (Knuth): s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// Fast2Sum (Dekker), for |a| >= |b| or a == 0: s + e == a + b exactly.
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
// TwoProduct through a fused multiply-add: p + e == a * b exactly.
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
// Whether hi (the float nearest hi + lo) is at least `margin` ulps away
// from the rounding midpoint on lo's side, i.e. |lo| <= (1/2 - margin) ulp
// with the ulp of that side.
__device__ __forceinline__ bool clear_of_midpoint(float hi, float lo, float half_minus_margin) {
  const uint32_t b = __float_as_uint(hi);
  const float u = lo < 0.0f ? hi - __uint_as_float(b - 1) : __uint_as_float(b + 1) - hi;
  return fabsf(lo) <= half_minus_margin * u;
}

// 2^(j/64), j = 0..63, as float pairs hi + lo (hi the nearest float, lo the
// nearest float to the rest; |error| < 2^-47 relative), for exp_ff.
__device__ static const uint32_t kExp2TabHi[64] = {
    0x3f800000, 0x3f8164d2, 0x3f82cd87, 0x3f843a29, 0x3f85aac3, 0x3f871f62,
    0x3f88980f, 0x3f8a14d5, 0x3f8b95c2, 0x3f8d1adf, 0x3f8ea43a, 0x3f9031dc,
    0x3f91c3d3, 0x3f935a2b, 0x3f94f4f0, 0x3f96942d, 0x3f9837f0, 0x3f99e046,
    0x3f9b8d3a, 0x3f9d3eda, 0x3f9ef532, 0x3fa0b051, 0x3fa27043, 0x3fa43516,
    0x3fa5fed7, 0x3fa7cd94, 0x3fa9a15b, 0x3fab7a3a, 0x3fad583f, 0x3faf3b79,
    0x3fb123f6, 0x3fb311c4, 0x3fb504f3, 0x3fb6fd92, 0x3fb8fbaf, 0x3fbaff5b,
    0x3fbd08a4, 0x3fbf179a, 0x3fc12c4d, 0x3fc346cd, 0x3fc5672a, 0x3fc78d75,
    0x3fc9b9be, 0x3fcbec15, 0x3fce248c, 0x3fd06334, 0x3fd2a81e, 0x3fd4f35b,
    0x3fd744fd, 0x3fd99d16, 0x3fdbfbb8, 0x3fde60f5, 0x3fe0ccdf, 0x3fe33f89,
    0x3fe5b907, 0x3fe8396a, 0x3feac0c7, 0x3fed4f30, 0x3fefe4ba, 0x3ff28177,
    0x3ff5257d, 0x3ff7d0df, 0x3ffa83b3, 0x3ffd3e0c,
};
__device__ static const uint32_t kExp2TabLo[64] = {
    0x00000000, 0xb1c43fd0, 0xb34ea7a9, 0xb2f14c87, 0x334f9891, 0xb352c2e6,
    0xb37eda4b, 0x336a92de, 0xb260aba1, 0x3336fcb7, 0xb3697465, 0x330628cd,
    0x33675624, 0x32bc4f9c, 0xb32e0212, 0x32dc8061, 0x33231b71, 0xb359be90,
    0xb30c5563, 0xb331a601, 0x33412342, 0x31fb9715, 0x30c3125a, 0xb323ec33,
    0xb32c9d5e, 0xb3162d36, 0xb3162b08, 0xb314ad82, 0xb22deaf6, 0xb3252deb,
    0xb37c5aa8, 0x32154889, 0x32cfe77a, 0xb266b974, 0x330ec5f7, 0xb31bd983,
    0xb3414fe8, 0xb3130b1a, 0xb2d6663e, 0xb2976da2, 0x320aa837, 0xb2dd5119,
    0xb37323a2, 0xb006c6c2, 0x3228fc24, 0xb2944353, 0xb35c1daa, 0xb3286024,
    0xb2d4a58a, 0xb2f61d41, 0xb3504a1c, 0xb37b43e3, 0xb21eab59, 0x33657d15,
    0xb2441be6, 0x33207898, 0xb24116de, 0x3276cca1, 0xb348464a, 0x32f167ff,
    0x32292436, 0x336615a2, 0xb2923758, 0x31cf486c,
};

// e^x in float-float arithmetic for -87 <= x <= 88, by Tang's table-driven
// method ("Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15(2), 1989): x = (64 m + j) ln2/64
// + r with |r| <= ln2/128, ln2/64 split in three parts (the first two with
// 11 significant bits, so k times them is exact), e^r = 1 + r + q with q
// the degree-5 Taylor tail, then e^x = 2^m (T_j + T_j (r + q)). The pair
// hi + lo is within 2^-36 of e^x (relative). Returns false, leaving `out`
// alone, outside that range or when the result would lie within 0.02 ulp of
// a rounding midpoint; otherwise `out` is e^x correctly rounded.
__device__ __forceinline__ bool exp_ff(float x, float& out) {
  if (!(x >= -87.0f && x <= 88.0f)) return false;
  const float kf = rintf(x * __uint_as_float(0x42b8aa3bu));  // 64/ln2
  const int k = (int)kf;
  const int j = k & 63;
  const int m = k >> 6;  // floor(k / 64)
  const float t = fmaf(-kf, __uint_as_float(0x3c318000u), x);  // exact
  const float p2 = kf * __uint_as_float(0xb65e8000u);          // exact
  float r_hi, r_lo;
  two_sum(t, -p2, r_hi, r_lo);
  r_lo = fmaf(-kf, __uint_as_float(0xae02e308u), r_lo);
  // q = r^2/2 + r^3/6 + r^4/24 + r^5/120, plus the cross term r_hi r_lo
  float q = fmaf(r_hi, __uint_as_float(0x3c088889u), __uint_as_float(0x3d2aaaabu));
  q = fmaf(q, r_hi, __uint_as_float(0x3e2aaaabu));
  q = fmaf(q, r_hi, 0.5f);
  q = q * (r_hi * r_hi);
  q = fmaf(r_hi, r_lo, q);
  float s_hi, s_lo;
  two_sum(r_hi, r_lo + q, s_hi, s_lo);
  const float T_hi = __uint_as_float(kExp2TabHi[j]), T_lo = __uint_as_float(kExp2TabLo[j]);
  float p, pe, y_hi, y_lo;
  two_prod(T_hi, s_hi, p, pe);
  two_sum(T_hi, p, y_hi, y_lo);
  y_lo = y_lo + ((T_lo + pe) + fmaf(T_hi, s_lo, T_lo * s_hi));
  fast_two_sum(y_hi, y_lo, y_hi, y_lo);
  if (!clear_of_midpoint(y_hi, y_lo, 0.48f)) return false;
  out = y_hi * __uint_as_float((uint32_t)(m + 127) << 23);  // 2^m, -126 <= m <= 126
  return true;
}

// The reference's std::exp(float) (source/wind.hpp:50), i.e. the C library
// expf, bit for bit: the double exponential rounded once to float is the
// correctly rounded value; only when it lies within 1% of an ulp of a
// rounding midpoint can the C library (about 0.502 ulp accurate) differ, and
// the build-time list of such arguments (c.expf_x, from the C library
// itself) gives the one-ulp correction.
__device__ __forceinline__ float exp_libm_dp(float x, const Consts& c) {
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

// The same value, first through exp_ff: where that returns a result it is
// the correctly rounded e^x and at least 0.02 ulp (less the two methods'
// errors, far below 0.01 ulp) clear of a midpoint, so exp_libm_dp would
// take no correction and round the double exponential to the same float;
// elsewhere (about 4% of arguments) exp_libm_dp runs. Single-precision
// float-float work instead of double precision, which is slow on this GPU.
__device__ __forceinline__ float exp_libm(float x, const Consts& c) {
  float r;
  if (exp_ff(x, r)) return r;
  return exp_libm_dp(x, c);
}

// (float)(1.0 - 0.3 * (double)s), the drag factor of Wind::fly
// (wind.hpp:87: glm multiplies the speed by a double). For 0 <= s < 2 the
// exact value 1 - 0.3d s (0.3d = Dhi + Dlo + 2^-52.4) is formed in float-
// float arithmetic within 2^-47, and its nearest float is returned when it
// lies more than 0.001 ulp (>= 2^-35) from a rounding midpoint: the double
// expression is within 2^-52 of the exact value, so it rounds to the same
// float. Otherwise the double expression is evaluated as written.
__device__ __forceinline__ float drag_factor(float s) {
  if (s >= 0.0f && s < 2.0f) {
    float p1, e1, a, b;
    two_prod(s, __uint_as_float(0x3e99999au), p1, e1);  // s * Dhi
    const float p2 = s * __uint_as_float(0xb24ccccdu);    // s * Dlo
    two_sum(1.0f, -p1, a, b);
    b = (b - e1) - p2;
    fast_two_sum(a, b, a, b);
    if (clear_of_midpoint(a, b, 0.499f)) return a;
  }
  return (float)(1.0 - 0.3 * (double)s);
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
