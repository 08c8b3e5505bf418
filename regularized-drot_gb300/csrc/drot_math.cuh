// drot_math.cuh -- correctly rounded division by a loop-invariant divisor.
//
// The QR prox divides every element by the same divisor kappa.  The
// reference evaluates max(v, 0.) / scale in double and stores the float
// result, i.e. the correctly rounded float quotient (double rounding is
// harmless for a quotient of two floats: 53 >= 2*24 + 2).  The IEEE float
// division instruction sequence costs a range check and a branch per
// element; this file instead uses Markstein's residual correction
// (P. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Dev. 34(1), 1990; restated as the
// "Markstein theorem" in Muller et al., Handbook of Floating-Point
// Arithmetic): with y = RN(1/b) and a quotient q within one ulp of a/b, the
// residual r = a - b*q is exact under an FMA and RN(q + r*y) = RN(a/b).
//
//   q0 = RN(a*y)              within 1.5 ulp
//   q1 = RN(q0 + RN(a-b*q0)*y) within 1 ulp (the first correction)
//   q2 = RN(q1 + RN(a-b*q1)*y) correctly rounded (the theorem)
//
// The theorem needs the residuals to stay in the normal range; inputs below
// 2^-90 (never produced by the DROT iterates, whose entries are sums of
// O(1/(m n)) terms) take the plain division instead.  Exhaustive checks over
// a full binade of a for several divisors are in tests/test_division.py.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define DROT_HD __host__ __device__ __forceinline__
#else
#define DROT_HD inline
#endif

namespace drot {

// Smallest dividend handled by the FMA sequence (2^-90).
constexpr float kDivTiny = 8.0779356e-28f;

// Bit pattern of kDivTiny minus one: a float t >= 0 with
// (uint32)(bits(t) - 1) < kDivTinyBitsM1 is a nonzero dividend below 2^-90.
constexpr unsigned kDivTinyBitsM1 = 0x12800000u - 1u;

// The FMA sequence alone: a / b correctly rounded for a == 0 or
// |a| >= 2^-90, b > 0 finite, y == RN(1/b).
DROT_HD float div_rn_by_fma(float a, float b, float y) {
  const float q0 = a * y;
  const float r0 = fmaf(-b, q0, a);
  const float q1 = fmaf(r0, y, q0);
  const float r1 = fmaf(-b, q1, a);
  return fmaf(r1, y, q1);
}

// a / b correctly rounded, for b > 0 finite and y == RN(1/b).  Zero takes
// the FMA path too (every step is exact); only nonzero dividends below 2^-90
// use the plain division.
DROT_HD float div_rn_by(float a, float b, float y) {
  if (a != 0.0f && fabsf(a) < kDivTiny) {
    return a / b;
  }
  return div_rn_by_fma(a, b, y);
}

}  // namespace drot

namespace drot {

// Error-free sum: s + e == a + b exactly (Knuth's TwoSum).
DROT_HD void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Group-lasso shrink factor max(1 - lambda / (sqrt(ns) + 1e-9), 0).
//
// The reference evaluates it in double from a float norm
// (core/kernel_glr.hpp:125, 320).  FP64 is a slow pipe on this part, so the
// quotient is carried as an unevaluated float pair (about 44 bits): the
// float result equals the rounded double one except when the exact value
// lies within 2^-44 of a rounding boundary.  The norm itself is a float
// sum, as in the reference, so that is below the rounding already present.
DROT_HD float gl_shrink(float ns, float lambda) {
  constexpr float kEpsHi = 1e-9f;
  constexpr float kEpsLo = (float)(1e-9 - (double)1e-9f);
  const float u = sqrtf(ns);
  float dh, dl;
  two_sum(u, kEpsHi, dh, dl);
  dl += kEpsLo;
  const float t = dh + dl;  // renormalise (dh, dl)
  dl = dl - (t - dh);
  dh = t;
  const float q1 = lambda / dh;
  if (!(q1 < 2.0f)) return 0.0f;  // 1 - w < 0 (also covers lambda/0)
  const float r = fmaf(-q1, dh, lambda) - q1 * dl;  // lambda - q1*d
  const float q2 = r / dh;
  float sh, sl;
  two_sum(1.0f, -q1, sh, sl);  // exact; sl == 0 when q1 >= 0.5
  const float v = sh + (sl - q2);
  return v > 0.0f ? v : 0.0f;
}

}  // namespace drot
