// Host check of the float-pair sums and of the squared-residual stop
// threshold (drot_math.cuh), compiled with the host compiler.
//
// 1. res2_threshold: for random eps and squared residuals r2 around eps^2
//    (including the threshold itself and its neighbours), r2 < T must agree
//    with sqrt(r2) < eps (strict) and sqrt(r2) <= eps (non-strict).
// 2. fp_add / fp_sqr: sums of n random terms, folded in the kernels' orders
//    (sequential per lane, then a butterfly tree), against a long double
//    reference; prints the largest relative error seen.
//
// Output: "<threshold mismatches> <max relative error of the pair sums>".
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <random>
#include <vector>

#include "drot_math.cuh"

using drot::fpair;

static long check_threshold(std::mt19937_64& rng) {
  std::uniform_real_distribution<double> ue(-30.0, 2.0);
  long bad = 0;
  for (int k = 0; k < 20000; ++k) {
    const float eps = (float)pow(10.0, ue(rng));
    for (int strict = 0; strict < 2; ++strict) {
      const double T = drot::res2_threshold(eps, strict != 0);
      const double e = (double)eps;
      double cands[7] = {T, nextafter(T, 0.0), nextafter(T, INFINITY), e * e,
                         nextafter(e * e, 0.0), nextafter(e * e, INFINITY), 0.0};
      std::uniform_real_distribution<double> ur(0.5, 1.5);
      for (int r = 0; r < 8; ++r) {
        const double r2 = r < 7 ? cands[r] : e * e * ur(rng);
        const bool want = strict ? sqrt(r2) < e : sqrt(r2) <= e;
        if ((r2 < T) != want) ++bad;
      }
    }
  }
  // Edge values: eps = 0, negative, huge.
  if (0.0 < drot::res2_threshold(0.0f, true)) ++bad;                 // sqrt(r2) < 0: never
  if (!(0.0 < drot::res2_threshold(0.0f, false))) ++bad;             // r2 == 0 stops
  if (drot::res2_threshold(0.0f, false) > 1e-300) ++bad;
  if (!(drot::res2_threshold(-1.0f, false) < 0.0)) ++bad;
  if (!(1e70 < drot::res2_threshold(3.0e38f, true))) ++bad;
  return bad;
}

static double check_sums(std::mt19937_64& rng) {
  double worst = 0.0;
  std::uniform_real_distribution<float> uf(0.0f, 1.0f);
  std::uniform_real_distribution<float> us(-1.0f, 1.0f);
  for (int trial = 0; trial < 200; ++trial) {
    const int lanes = 32;
    const int per = 1 + (int)(rng() % 4000);
    const bool squares = trial % 2 == 1;
    std::vector<fpair> lane(lanes, fpair{0.0f, 0.0f});
    long double ref = 0.0L;
    for (int l = 0; l < lanes; ++l) {
      float hi = 0.0f, lo = 0.0f;
      for (int i = 0; i < per; ++i) {
        const float v = squares ? us(rng) * 1e-3f : uf(rng) * 1e-6f;
        if (squares) {
          lane[l] = drot::fp_add(lane[l], drot::fp_sqr(v));
          ref += (long double)v * (long double)v;
        } else {
          float e;
          drot::two_sum(hi, v, hi, e);  // the per-lane TwoSum carry of the kernels
          lo += e;
          ref += (long double)v;
        }
      }
      if (!squares) lane[l] = fpair{hi, lo};
    }
    // Butterfly as in warp_sum_fp (lane 0's view).
    for (int o = 16; o > 0; o >>= 1) {
      std::vector<fpair> nxt(lanes);
      for (int l = 0; l < lanes; ++l) nxt[l] = drot::fp_add(lane[l], lane[l ^ o]);
      lane = nxt;
    }
    const long double got = (long double)lane[0].hi + (long double)lane[0].lo;
    const double rel = (double)fabsl((got - ref) / ref);
    if (rel > worst) worst = rel;
  }
  return worst;
}

int main() {
  std::mt19937_64 rng(12345);
  const long bad = check_threshold(rng);
  const double worst = check_sums(rng);
  printf("%ld %.3e\n", bad, worst);
  return bad == 0 ? 0 : 1;
}
