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

// Float-pair ("double-float") sums for the per-iteration reductions (mass,
// objective, squared residual).  A pair (hi, lo) stands for hi + lo with
// |lo| <= ulp(hi)/2 after fp_add; sums of n terms carry about 44 bits, which
// is more than the reference's float sums (core/kernel_qr.hpp:92-111, 432-440)
// and, unlike FP64 -- a narrow pipe on this part -- run on the FP32 units.
struct fpair {
  float hi, lo;
};

DROT_HD fpair fp_make(float v) { return fpair{v, 0.0f}; }

// Sum of two pairs (TwoSum of the heads, tails added, Fast2Sum renormalise).
DROT_HD fpair fp_add(fpair a, fpair b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  const float h = s + e;
  return fpair{h, e - (h - s)};
}

// Exact square v*v as a pair (TwoProduct with one fma).
DROT_HD fpair fp_sqr(float v) {
#ifdef __CUDA_ARCH__
  const float p = __fmul_rn(v, v);  // not contracted into the fma below
  return fpair{p, __fmaf_rn(v, v, -p)};
#else
  const float p = v * v;
  return fpair{p, fmaf(v, v, -p)};
#endif
}

DROT_HD double fp_value(fpair a) { return (double)a.hi + (double)a.lo; }

// The device tests the squared residual r2 (FP64) against one threshold T:
// sqrt(r2) < eps (strict, QR) or sqrt(r2) <= eps (GL, numpy-API loop) holds
// exactly when r2 < T, with T the smallest double whose correctly rounded
// square root is >= eps (strict) or > eps.  sqrt is monotonic, so T is found
// by stepping from eps^2 one ulp at a time (a few steps at most).
inline double res2_threshold(float eps_f, bool strict) {
  const double e = (double)eps_f;
  if (!(e >= 0.0)) return -1.0;              // eps < 0 or NaN: never stop
  if (isinf(e)) return INFINITY;             // every finite residual stops
  auto ok = [&](double t) { return strict ? sqrt(t) >= e : sqrt(t) > e; };
  double t = e * e;
  while (t > 0.0 && ok(nextafter(t, 0.0))) t = nextafter(t, 0.0);
  while (!ok(t)) t = nextafter(t, INFINITY);
  return t;
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
