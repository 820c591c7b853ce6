// GELU and its derivative for the surrogate's kernels.
//
// GELU(v) = v Phi(v), Phi the standard normal CDF. Phi comes from the
// complementary error function by Abramowitz & Stegun, Handbook of
// Mathematical Functions, formula 7.1.26: for z >= 0,
//   erfc(z) = t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) exp(-z^2) + e(z),
//   t = 1 / (1 + p z), |e(z)| <= 1.5e-7,
// so Phi(-|v|) = erfc(|v| / sqrt 2) / 2 and Phi(|v|) = 1 - Phi(-|v|); the
// tail side is formed without cancellation. The reciprocal and exp(-z^2)
// use the hardware approximations (a few ulp), far inside the bf16 rounding
// of the results (2^-8 relative). exp(-z^2) = exp(-v^2 / 2) also gives the
// Gaussian density that the derivative needs:
//   GELU'(v) = Phi(v) + v exp(-v^2 / 2) / sqrt(2 pi).
#pragma once

namespace swe {

struct NormalCdf {
  float cdf;    // Phi(v)
  float gauss;  // exp(-v^2 / 2)
};

__device__ __forceinline__ NormalCdf normal_cdf(float v) {
  const float z = fabsf(v) * 0.70710678118654752f;
  const float t = __fdividef(1.0f, fmaf(0.3275911f, z, 1.0f));
  float p = fmaf(t, 1.061405429f, -1.453152027f);
  p = fmaf(t, p, 1.421413741f);
  p = fmaf(t, p, -0.284496736f);
  p = fmaf(t, p, 0.254829592f);
  const float g = __expf(-(z * z));
  const float tail = 0.5f * (p * t) * g;  // Phi(-|v|)
  return NormalCdf{v >= 0.0f ? 1.0f - tail : tail, g};
}

__device__ __forceinline__ float gelu_as(float v) { return v * normal_cdf(v).cdf; }

__device__ __forceinline__ float gelu_grad_as(float v) {
  const NormalCdf n = normal_cdf(v);
  return n.cdf + v * 0.3989422804014327f * n.gauss;
}

}  // namespace swe
