// Per-point likelihood terms for the Laplace path.
//
//  * PGB_LIK_GAUSSIAN: log N(y; f, sigma^2), restating log_gaussian_likelihood
//    / norm_logpdf (utilities.py:60-61,64-70).
//  * PGB_LIK_PROBIT: log(Phi(z2) - Phi(z1) + 1e-10) with z_k = (b_k - f)/sigma,
//    Phi through erf and the +-inf cutpoint guards, restating
//    log_probit_likelihood / probit / norm_cdf (utilities.py:31-34,47-57,
//    195-229).  The f-derivatives are those JAX autodiff gives for that
//    expression (approximators.py:92-95).
//  * PGB_LIK_PROBIT_STABLE: the same model with log P and its ratios
//    evaluated through erfcx Mills ratios (no +1e-10), so tails far from
//    the data stay finite and accurate.
//
// Derivatives are built from G(z1, z2) = log P:
//   G_1 = -phi(z1)/P, G_2 = phi(z2)/P,
//   G_11 = -z1 G_1 - G_1^2, G_22 = -z2 G_2 - G_2^2, G_12 = -G_1 G_2,
//   and the third partials obtained by differentiating those once more,
// then mapped to f, sigma and the two cutpoints with dz_k/df = -1/sigma,
// dz_k/db_k = 1/sigma, dz_k/dsigma = -z_k/sigma.  A side whose cutpoint is
// infinite has G_k = 0 and its z_k is replaced by 0 so no inf*0 arises.
#pragma once

#include "common.cuh"

namespace pgb {

constexpr float kSqrt2 = 1.41421356237309504880f;
constexpr float kOverSqrt2Pi = 0.39894228040143267794f;
constexpr float kLogOverSqrt2Pi = -0.91893853320467274178f;
constexpr float kProbitEps = 1e-10f;
constexpr float kSqrt2OverPi = 0.79788456080286535588f;

struct LikOut {
  float logp, d1, d2, d3;
  // partials in (sigma, b_lo, b_hi) of logp, d1, d2 (gradient only)
  float lp_s, d1_s, d2_s;
  float lp_lo, d1_lo, d2_lo;
  float lp_hi, d1_hi, d2_hi;
  int ylo;  // index of the lower cutpoint (class y); -1 for Gaussian
};

__device__ __forceinline__ float ndtr_ref(float z) {
  // 0.5 * (1 + erf(z / sqrt 2)), utilities.py:18-19
  return 0.5f * (1.0f + erff(z / kSqrt2));
}

template <bool WANT_PARTIALS>
__device__ __forceinline__ void lik_point(int lik, float f, float yv, int yi, float sig,
                                          const float* __restrict__ cut, LikOut& o) {
  if (lik == PGB_LIK_GAUSSIAN) {
    const float z = (f - yv) / sig;
    const float s2 = sig * sig;
    o.logp = kLogOverSqrt2Pi - z * z / 2.0f - logf(sig);
    o.d1 = (yv - f) / s2;
    o.d2 = -1.0f / s2;
    o.d3 = 0.0f;
    o.ylo = -1;
    if (WANT_PARTIALS) {
      o.lp_s = (z * z - 1.0f) / sig;
      o.d1_s = -2.0f * (yv - f) / (s2 * sig);
      o.d2_s = 2.0f / (s2 * sig);
      o.lp_lo = o.d1_lo = o.d2_lo = o.lp_hi = o.d1_hi = o.d2_hi = 0.0f;
    }
    return;
  }
  const float blo = __ldg(cut + yi);
  const float bhi = __ldg(cut + yi + 1);
  const bool fin1 = isfinite(blo);
  const bool fin2 = isfinite(bhi);
  float z1 = fin1 ? (blo - f) / sig : 0.0f;
  float z2 = fin2 ? (bhi - f) / sig : 0.0f;
  float G1, G2;
  o.logp = 0.0f;
  if (lik == PGB_LIK_PROBIT) {
    const float c1 = fin1 ? ndtr_ref(z1) : 0.0f;
    const float c2 = fin2 ? ndtr_ref(z2) : 1.0f;
    const float pe = (c2 - c1) + kProbitEps;
    o.logp = logf(pe);
    const float p1 = kOverSqrt2Pi * expf(-0.5f * z1 * z1);
    const float p2 = kOverSqrt2Pi * expf(-0.5f * z2 * z2);
    G1 = fin1 ? -p1 / pe : 0.0f;
    G2 = fin2 ? p2 / pe : 0.0f;
  } else {
    // stable: one-sided intervals through Mills ratios
    //   lambda(z) = phi(z) / Q(z) = sqrt(2/pi) / erfcx(z / sqrt 2),
    // with rho = Q(z2) / Q(z1) (upper side) or Phi(z1) / Phi(z2) (lower
    // side) formed from erfcx ratios, so no exp of a large log difference
    // is taken and G_1, G_2 keep float32 relative accuracy in the tails.
    if (fin1 && z1 >= 0.0f) {
      const float e1 = erfcxf(z1 / kSqrt2);
      const float rho = fin2 ? (erfcxf(z2 / kSqrt2) / e1) * expf(-0.5f * (z2 - z1) * (z2 + z1)) : 0.0f;
      o.logp = logf(0.5f * e1) - 0.5f * z1 * z1 + log1pf(-rho);
      const float l1 = kSqrt2OverPi / e1;
      G1 = -l1 / (1.0f - rho);
      G2 = fin2 ? (kSqrt2OverPi / erfcxf(z2 / kSqrt2)) * rho / (1.0f - rho) : 0.0f;
    } else if (fin2 && z2 <= 0.0f) {
      const float e2 = erfcxf(-z2 / kSqrt2);
      const float rho = fin1 ? (erfcxf(-z1 / kSqrt2) / e2) * expf(-0.5f * (z1 - z2) * (z1 + z2)) : 0.0f;
      o.logp = logf(0.5f * e2) - 0.5f * z2 * z2 + log1pf(-rho);
      G2 = (kSqrt2OverPi / e2) / (1.0f - rho);
      G1 = fin1 ? -(kSqrt2OverPi / erfcxf(-z1 / kSqrt2)) * rho / (1.0f - rho) : 0.0f;
    } else {
      // z1 < 0 < z2 (or an infinite side): P >= 0 is a sum of moderate terms
      const float lo = fin1 ? 0.5f * erfcf(-z1 / kSqrt2) : 0.0f;   // Phi(z1)
      const float hi = fin2 ? 0.5f * erfcf(z2 / kSqrt2) : 0.0f;    // Q(z2)
      const float P = 1.0f - (lo + hi);
      o.logp = log1pf(-(lo + hi));
      G1 = fin1 ? -kOverSqrt2Pi * expf(-0.5f * z1 * z1) / P : 0.0f;
      G2 = fin2 ? kOverSqrt2Pi * expf(-0.5f * z2 * z2) / P : 0.0f;
    }
  }
  const float G11 = -z1 * G1 - G1 * G1;
  const float G22 = -z2 * G2 - G2 * G2;
  const float G12 = -G1 * G2;
  const float G111 = -G1 - z1 * G11 - 2.0f * G1 * G11;
  const float G112 = -z1 * G12 - 2.0f * G1 * G12;
  const float G122 = -z2 * G12 - 2.0f * G2 * G12;
  const float G222 = -G2 - z2 * G22 - 2.0f * G2 * G22;
  const float is = 1.0f / sig;
  const float is2 = is * is, is3 = is2 * is;
  const float S2 = G11 + 2.0f * G12 + G22;
  const float dS1 = G111 + 2.0f * G112 + G122;
  const float dS2 = G112 + 2.0f * G122 + G222;
  o.d1 = -(G1 + G2) * is;
  o.d2 = S2 * is2;
  o.d3 = -(G111 + 3.0f * G112 + 3.0f * G122 + G222) * is3;
  o.ylo = yi;
  if (WANT_PARTIALS) {
    o.lp_s = -(z1 * G1 + z2 * G2) * is;
    o.d1_s = (z1 * (G11 + G12) + z2 * (G12 + G22) + G1 + G2) * is2;
    o.d2_s = -(z1 * dS1 + z2 * dS2 + 2.0f * S2) * is3;
    o.lp_lo = G1 * is;
    o.d1_lo = -(G11 + G12) * is2;
    o.d2_lo = dS1 * is3;
    o.lp_hi = G2 * is;
    o.d1_hi = -(G12 + G22) * is2;
    o.d2_hi = dS2 * is3;
  }
}

}  // namespace pgb
