// Host check of drot::gl_shrink against the reference's double formula
// (float)max(1. - lambda / ((double)sqrtf(ns) + 1e-9), 0.).
// Prints: samples, exact matches, mismatches of 1 ulp, larger mismatches.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "drot_math.cuh"

static float ref_shrink(float ns, float lambda) {
  const double sh = 1.0 - (double)lambda / ((double)sqrtf(ns) + 1e-9);
  return (float)(sh > 0.0 ? sh : 0.0);
}

static int32_t ulp_dist(float a, float b) {
  int32_t ia, ib;
  std::memcpy(&ia, &a, 4);
  std::memcpy(&ib, &b, 4);
  return ia > ib ? ia - ib : ib - ia;
}

int main() {
  uint64_t s = 0x243f6a8885a308d3ull;
  long n = 0, exact = 0, one = 0, more = 0;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  for (int i = 0; i < (1 << 23); ++i) {
    // norms^2 over 1e-30 .. 1e2, lambda over 1e-8 .. 1e-1, and lambda near sqrt(ns)
    const double e1 = -30.0 + 32.0 * (double)(rnd() % 1000000) / 1e6;
    const float ns = (float)std::pow(10.0, e1);
    float lambda;
    if (i & 1) {
      lambda = (float)std::pow(10.0, -8.0 + 7.0 * (double)(rnd() % 1000000) / 1e6);
    } else {
      lambda = (float)(std::sqrt((double)ns) * (0.9 + 0.2 * (double)(rnd() % 1000000) / 1e6));
    }
    const float a = drot::gl_shrink(ns, lambda), b = ref_shrink(ns, lambda);
    ++n;
    const int32_t d = ulp_dist(a, b);
    if (d == 0) ++exact; else if (d == 1) ++one; else ++more;
  }
  const float zs[] = {0.0f, 1e-40f};
  for (float z : zs) {
    ++n;
    if (drot::gl_shrink(z, 1e-3f) == ref_shrink(z, 1e-3f)) ++exact; else ++more;
    ++n;
    if (drot::gl_shrink(z, 0.0f) == ref_shrink(z, 0.0f)) ++exact; else ++more;
  }
  std::printf("%ld %ld %ld %ld\n", n, exact, one, more);
  return more ? 1 : 0;
}
