// Host check of athg_numeric.h: the integer format conversions against the host's own
// IEEE 754 casts, and the error-free sums against exact (long double / double) sums.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include "athg_numeric.h"

using namespace athg;

static int fails = 0;
#define CHECK(c, ...) do { if (!(c)) { if (fails++ < 10) { std::printf(__VA_ARGS__); std::printf("\n"); } } } while (0)

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
  std::mt19937_64 rng(12345);
  // binary32 -> binary64: every normal float, sampled across all bit patterns
  for (long t = 0; t < n; ++t) {
    uint32_t u = (uint32_t)rng();
    float f = from_bits_f(u);
    double got = f2d_int(f);
    uint32_t a = u & 0x7fffffffu;
    if (a >= 0x00800000u && a < 0x7f800000u) {
      CHECK(bits_d(got) == bits_d((double)f), "f2d %08x", u);
    } else if (a < 0x00800000u) {
      CHECK(got == 0.0 && std::signbit(got) == std::signbit(f), "f2d subnormal %08x", u);
    } else if (a == 0x7f800000u) {
      CHECK(std::isinf(got) && std::signbit(got) == std::signbit(f), "f2d inf %08x", u);
    } else {
      CHECK(std::isnan(got), "f2d nan %08x", u);
    }
  }
  // binary64 -> binary32, round to nearest even
  std::uniform_int_distribution<int> ex(-140, 140);
  for (long t = 0; t < n; ++t) {
    double d;
    int kind = (int)(t % 4);
    if (kind == 0) {
      d = std::ldexp((double)(rng() >> 11) / 9007199254740992.0 + 0.5, ex(rng));
    } else if (kind == 1) {  // exact ties between two binary32 values
      uint64_t b = bits_d(std::ldexp(1.0 + (double)(rng() >> 40) / 16777216.0, ex(rng) % 120));
      b = (b & ~0x1fffffffull) | 0x10000000ull;
      d = from_bits_d(b);
    } else if (kind == 2) {  // one ulp either side of a tie
      uint64_t b = bits_d(std::ldexp(1.0 + (double)(rng() >> 40) / 16777216.0, ex(rng) % 120));
      b = (b & ~0x1fffffffull) | 0x10000000ull;
      b += (rng() & 1) ? 1 : -1;
      d = from_bits_d(b);
    } else {
      d = from_bits_d(rng());
    }
    if (rng() & 1) d = -d;
    float got = d2f_int(d);
    float ref = (float)d;
    if (std::isnan(d)) {
      CHECK(std::isnan(got), "d2f nan");
    } else if (ref != 0.0f && std::fabs(ref) < 1.1754943508222875e-38f) {
      CHECK(got == 0.0f && std::signbit(got) == std::signbit(d), "d2f subnormal %a", d);
    } else if (ref == 0.0f) {
      CHECK(got == 0.0f, "d2f zero %a", d);
    } else {
      CHECK(bits_f(got) == bits_f(ref), "d2f %a -> %a want %a", d, (double)got, (double)ref);
    }
  }
  // TwoSum and the cascaded sums
  std::normal_distribution<double> nd(0.0, 1.0);
  double worst3 = 0.0, worst2 = 0.0;
  for (long t = 0; t < n / 4; ++t) {
    float x[6];
    double scale = std::ldexp(1.0, ex(rng) % 40);
    for (int q = 0; q < 6; ++q) x[q] = (float)(scale * nd(rng) * ((q & 1) ? 1.0 : (1.0 + 1e-3 * nd(rng))));
    float s, e;
    two_sum(x[0], x[1], s, e);
    CHECK((long double)s + e == (long double)x[0] + x[1], "two_sum");
    float hi, lo;
    sum3diff(x[0], x[1], x[2], x[3], x[4], x[5], hi, lo);
    long double ex3 = ((long double)x[0] - x[1]) + ((long double)x[2] - x[3]) + ((long double)x[4] - x[5]);
    long double mag = 0;
    for (int q = 0; q < 6; ++q) mag += std::fabs((long double)x[q]);
    double r3 = (double)(std::fabs((long double)hi + lo - ex3) / mag);
    if (r3 > worst3) worst3 = r3;
    sum2diff(x[0], x[1], x[2], x[3], hi, lo);
    long double ex2 = ((long double)x[0] - x[1]) + ((long double)x[2] - x[3]);
    mag = std::fabs((long double)x[0]) + std::fabs((long double)x[1]) + std::fabs((long double)x[2]) +
          std::fabs((long double)x[3]);
    double r2 = (double)(std::fabs((long double)hi + lo - ex2) / mag);
    if (r2 > worst2) worst2 = r2;
  }
  CHECK(worst3 <= std::ldexp(1.0, -44), "sum3diff error %g", worst3);
  CHECK(worst2 <= std::ldexp(1.0, -45), "sum2diff error %g", worst2);
  std::printf("fails=%d worst3=%.3g worst2=%.3g\n", fails, worst3, worst2);
  return fails ? 1 : 0;
}
