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
  // division by an invariant: every d up to 2^17 against a spread of numerators (both ends
  // of the range, around multiples of d, random), and every a < 2^20 for a few d
  for (uint32_t d = 1; d <= (1u << 17); ++d) {
    const FastDiv f = fastdiv_make(d);
    const uint32_t hi = 0x7fffffffu;
    const uint32_t probe[8] = {0u, 1u, d - 1u, d, d + 1u, hi, hi - 1u, hi - (hi % d)};
    for (uint32_t a : probe)
      if (a <= hi) CHECK(fastdiv((int)a, f) == (int)(a / d), "fastdiv %u / %u", a, d);
    for (int r = 0; r < 16; ++r) {
      const uint32_t a = (uint32_t)(rng() & hi);
      CHECK(fastdiv((int)a, f) == (int)(a / d), "fastdiv %u / %u", a, d);
      const uint32_t q = a / d, b = q * d;  // around a multiple of d
      CHECK(fastdiv((int)b, f) == (int)q, "fastdiv %u / %u", b, d);
      if (b) CHECK(fastdiv((int)(b - 1), f) == (int)((b - 1) / d), "fastdiv %u / %u", b - 1, d);
    }
  }
  {
    const uint32_t ds[6] = {3, 7, 65, 69, 1000, 65537};
    for (uint32_t d : ds) {
      const FastDiv f = fastdiv_make(d);
      for (uint32_t a = 0; a < (1u << 20); ++a)
        CHECK(fastdiv((int)a, f) == (int)(a / d), "fastdiv %u / %u", a, d);
    }
  }
  // small-range quotients by an FP32 reciprocal: every a < 2^12, every b <= 2^10
  for (int b = 1; b <= 1024; ++b) {
    const float rb = 1.0f / (float)b;
    for (int a = 0; a < 4096; ++a) CHECK(div_small(a, rb) == a / b, "div_small %d / %d", a, b);
  }
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
  // double-float split and the primitive-recovery pressure p = (g-1)(E - m^2/(2d) - B^2/2)
  double worst_split = 0.0, worst_p = 0.0;
  std::uniform_real_distribution<double> ud01(0.0, 1.0);
  for (long t = 0; t < n / 4; ++t) {
    double x = std::ldexp(0.5 + ud01(rng), ex(rng) % 60) * ((rng() & 1) ? 1 : -1);
    ff sx = split_ff(x);
    double es = std::fabs((double)((long double)sx.hi + sx.lo - x)) / std::fabs(x);
    if (es > worst_split) worst_split = es;
    CHECK(bits_f(sx.hi) == bits_f((float)x), "split hi %a", x);
    // a cell: density, momenta, face fields (B = average of the two faces), energy with
    // internal energy down to 1e-6 of the kinetic + magnetic energy
    double d = std::ldexp(0.5 + ud01(rng), (int)(rng() % 20) - 10);
    double m[3], f[6];
    for (int q = 0; q < 3; ++q) m[q] = d * 3.0 * (ud01(rng) - 0.5);
    for (int q = 0; q < 6; ++q) f[q] = 2.0 * (ud01(rng) - 0.5);
    long double K = 0.5L * ((long double)m[0] * m[0] + (long double)m[1] * m[1] +
                            (long double)m[2] * m[2]) / d;
    long double M = 0.0L;
    for (int q = 0; q < 3; ++q) {
      long double bq = 0.5L * ((long double)f[2 * q] + f[2 * q + 1]);
      M += 0.5L * bq * bq;
    }
    double eint = (double)((K + M) * std::pow(10.0L, -6.0L * ud01(rng)));
    double E = (double)(K + M) + eint;
    const double gm1 = 2.0 / 3.0;
    long double pex = (long double)gm1 * ((long double)E - K - M);
    ff dd = split_ff(d), mm = ff_sqr(split_ff(m[0]));
    mm = ff_add(mm, ff_sqr(split_ff(m[1])));
    mm = ff_add(mm, ff_sqr(split_ff(m[2])));
    ff k2 = ff_mul(mm, ff_recip(dd));
    ff ss = ff_sqr(ff_add(split_ff(f[0]), split_ff(f[1])));
    ss = ff_add(ss, ff_sqr(ff_add(split_ff(f[2]), split_ff(f[3]))));
    ss = ff_add(ss, ff_sqr(ff_add(split_ff(f[4]), split_ff(f[5]))));
    ff xx = ff_add(k2, ff_scale(ss, 0.25f));
    ff pp = ff_mul(ff_sub(split_ff(E), ff_scale(xx, 0.5f)), split_ff(gm1));
    double ep = (double)(std::fabs((long double)pp.hi + pp.lo - pex) / (gm1 * (long double)E));
    if (ep > worst_p) worst_p = ep;
  }
  // the short path of split_ff gives the general routine's bits: random patterns across
  // every exponent, and the edges of its range (zeros, subnormals, infinities, NaNs and
  // the binary64 exponents 942..943 and 1142..1143 around 2^-80 and 2^120)
  for (long t = 0; t < n; ++t) {
    uint64_t u = rng();
    if (t % 3 == 1) {  // exponent near the range edges
      static const uint64_t eds[] = {0, 1, 941, 942, 943, 944, 1141, 1142, 1143, 1144, 2046, 2047};
      u = (u & 0x800fffffffffffffull) | (eds[rng() % 12] << 52);
    } else if (t % 3 == 2) {  // mantissas with ties and near-ties at the 29 dropped bits
      const uint64_t tail = (rng() & 3) == 0 ? 0x10000000ull : (rng() & 0x1fffffffull);
      u = (u & ~0x1fffffffull) | tail;
    }
    const double x = from_bits_d(u);
    const ff a = split_ff(x), g = split_ff_general(x);
    CHECK(bits_f(a.hi) == bits_f(g.hi) && bits_f(a.lo) == bits_f(g.lo),
          "split short path %016llx", (unsigned long long)u);
  }
  // seven-point sum 6c - sum(n) in 64-bit integers: smooth fields (neighbours within a
  // few percent of the centre, the multigrid's case, where FP64 cancels most digits),
  // independent values over many exponents, zeros and sign changes; against long double
  double worst_lap = 0.0;
  std::uniform_int_distribution<int> ex2(-60, 60);
  for (long t = 0; t < n / 4; ++t) {
    const int kind = (int)(t % 3);
    const double c = std::ldexp(0.5 + ud01(rng), ex2(rng)) * ((rng() & 1) ? 1 : -1);
    double nb[6];
    for (int q = 0; q < 6; ++q) {
      if (kind == 0) nb[q] = c * (1.0 + 0.05 * (ud01(rng) - 0.5));
      else if (kind == 1) nb[q] = std::ldexp(0.5 + ud01(rng), ex2(rng)) * ((rng() & 1) ? 1 : -1);
      else nb[q] = (q == (int)(rng() % 6)) ? 0.0 : c * (ud01(rng) - 0.5);
    }
    ff L;
    const bool ok = lap7_ff(c, nb, L);
    CHECK(ok, "lap7 refused %a", c);
    if (!ok) continue;
    long double ex = 6.0L * c, mag = 6.0L * std::fabs((long double)c), mx = std::fabs((long double)c);
    for (int q = 0; q < 6; ++q) {
      ex -= nb[q];
      mag += std::fabs((long double)nb[q]);
      if (std::fabs((long double)nb[q]) > mx) mx = std::fabs((long double)nb[q]);
    }
    const long double err = std::fabs((long double)L.hi + L.lo - ex);
    const long double bound = std::ldexp(1.0L, -46) * std::fabs(ex) + std::ldexp(1.0L, -54) * mx;
    CHECK(err <= bound, "lap7 error %Lg bound %Lg (c %a)", err, bound, c);
    const double rel = (double)(err / mag);
    if (rel > worst_lap) worst_lap = rel;
  }
  {
    const double inf = INFINITY, nan = NAN, z6[6] = {0, 0, 0, 0, 0, 0};
    const double in6[6] = {1.0, 1.0, inf, 1.0, 1.0, 1.0}, nn6[6] = {1.0, nan, 1.0, 1.0, 1.0, 1.0};
    ff L = {7.0f, 7.0f};
    CHECK(!lap7_ff(1.0, in6, L) && !lap7_ff(1.0, nn6, L) && !lap7_ff(0.0, z6, L) &&
              !lap7_ff(1e-30, z6, L) && !lap7_ff(1e40, z6, L) && L.hi == 7.0f,
          "lap7 outside its range must refuse and leave the result");
    const double small = 1e-20;
    CHECK(lap7_ff(small, z6, L) &&
              std::fabs((long double)L.hi + L.lo - 6.0L * small) <= std::ldexp(6.0L * small, -46),
          "lap7 small");
  }
  std::printf("lap7 worst error / (6|c| + sum|n|) = %.3g\n", worst_lap);
  CHECK(worst_split <= std::ldexp(1.0, -45), "split error %g", worst_split);
  CHECK(worst_p <= std::ldexp(1.0, -42), "pressure error %g", worst_p);
  std::printf("split=%.3g pressure(rel. to (g-1)E)=%.3g\n", worst_split, worst_p);
  CHECK(worst3 <= std::ldexp(1.0, -44), "sum3diff error %g", worst3);
  CHECK(worst2 <= std::ldexp(1.0, -45), "sum2diff error %g", worst2);
  std::printf("fails=%d worst3=%.3g worst2=%.3g\n", fails, worst3, worst2);
  return fails ? 1 : 0;
}
