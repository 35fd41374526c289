// Checks the integer-pipe conversions of csrc/convert.cuh (double <-> float,
// non-negative int -> double)
// against the C++ casts (IEEE round to nearest even) on random bit patterns,
// random values across the float range and the boundary cases.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <limits>
#include <random>

#include "convert.cuh"

using sph::bitsOfDouble;
using sph::bitsOfFloat;

static long bad = 0;

static void checkD(double x) {
  const float want = (float)x, got = sph::toFloatRN(x);
  if (bitsOfFloat(want) != bitsOfFloat(got) && !(std::isnan(want) && std::isnan(got))) {
    if (bad < 10) std::printf("toFloatRN(%a) = %a, cast %a\n", x, (double)got, (double)want);
    ++bad;
  }
}
static void checkF(float x) {
  const double want = (double)x, got = sph::toDouble(x);
  if (bitsOfDouble(want) != bitsOfDouble(got) && !(std::isnan(want) && std::isnan(got))) {
    if (bad < 10) std::printf("toDouble(%a) = %a, cast %a\n", (double)x, got, want);
    ++bad;
  }
}

int main() {
  std::mt19937_64 rng(12345);
  for (long k = 0; k < 4000000; ++k) {
    uint64_t b = rng();
    double x;
    std::memcpy(&x, &b, sizeof x);
    checkD(x);
    uint32_t f = (uint32_t)(b >> 17);
    float y;
    std::memcpy(&y, &f, sizeof y);
    checkF(y);
  }
  std::uniform_real_distribution<double> u(-130.0, 130.0);
  for (long k = 0; k < 4000000; ++k) {
    const double x = (k & 1 ? -1.0 : 1.0) * std::exp2(u(rng));
    checkD(x);
    checkF((float)x);
  }
  // ties and near-ties at every exponent, the normal/subnormal edge, FLT_MAX
  for (int e = -160; e <= 130; ++e) {
    const double base = std::ldexp(1.0, e);
    for (int m = 0; m < 64; ++m) {
      const double x = base * (1.0 + m * std::ldexp(1.0, -24)) ;
      for (const double d : {-1.0, 0.0, 1.0}) {
        const double y = x + d * std::ldexp(base, -53);
        checkD(y);
        checkD(-y);
        checkD(x + std::ldexp(base, -24));   // exact ties
      }
    }
  }
  const double specials[] = {0.0, -0.0, std::numeric_limits<double>::infinity(),
                             -std::numeric_limits<double>::infinity(), std::numeric_limits<double>::quiet_NaN(),
                             (double)std::numeric_limits<float>::max(), (double)std::numeric_limits<float>::min(),
                             std::numeric_limits<double>::max(), std::numeric_limits<double>::min(),
                             std::numeric_limits<double>::denorm_min()};
  for (const double x : specials) {
    checkD(x);
    checkD(-x);
    checkF((float)x);
  }
  for (int c = -3; c < 5000000; ++c) {
    const double want = (double)c, got = sph::smallIntToDouble(c);
    if (bitsOfDouble(want) != bitsOfDouble(got)) {
      if (bad < 10) std::printf("smallIntToDouble(%d) = %a\n", c, got);
      ++bad;
    }
  }
  for (int s = 0; s < 31; ++s)
    for (int d = -2; d <= 2; ++d) {
      const long long v = (1LL << s) + d;
      if (v < 0 || v > 0x7fffffff) continue;
      if (bitsOfDouble((double)v) != bitsOfDouble(sph::smallIntToDouble((int)v))) ++bad;
    }
  std::printf("%ld mismatches\n", bad);
  return bad == 0 ? 0 : 1;
}
