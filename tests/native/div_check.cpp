// Host check of drot::div_rn_by against IEEE float division.
// Usage: div_check <b> [<b> ...]
//   For each divisor b: every dividend a in [1, 2) (all 2^23 significands),
//   then 2^22 random dividends spread over [2^-90, 2^30].  Prints the
//   number of mismatches per divisor; exit status 1 if any.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "drot_math.cuh"

static float from_bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

int main(int argc, char** argv) {
  long total_bad = 0;
  for (int k = 1; k < argc; ++k) {
    const float b = std::strtof(argv[k], nullptr);
    const float y = (float)(1.0 / (double)b);
    long bad = 0;
    for (uint32_t m = 0; m < (1u << 23); ++m) {
      const float a = from_bits(0x3f800000u | m);
      if (drot::div_rn_by(a, b, y) != a / b) ++bad;
    }
    uint64_t s = 0x9e3779b97f4a7c15ull ^ (uint64_t)k;
    for (int i = 0; i < (1 << 22); ++i) {
      s ^= s << 13; s ^= s >> 7; s ^= s << 17;
      const uint32_t e = 37u + (uint32_t)(s % 120u);  // biased exponent of 2^-90 .. 2^30
      const float a = from_bits((e << 23) | (uint32_t)((s >> 20) & 0x7fffffu));
      if (drot::div_rn_by(a, b, y) != a / b) ++bad;
    }
    if (drot::div_rn_by(0.0f, b, y) != 0.0f) ++bad;
    std::printf("%.9g %ld\n", b, bad);
    total_bad += bad;
  }
  return total_bad ? 1 : 0;
}
