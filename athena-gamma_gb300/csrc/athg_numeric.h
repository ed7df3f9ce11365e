// athg_numeric.h -- format conversions and error-free sums of the mixed-precision path.
//
// FP64 instructions (conversions included) issue at a small fraction of the FP32 rate on
// this GPU, so the mixed path converts between the IEEE 754 binary32 and binary64 formats
// with integer operations and sums FP32 values with error-free transformations, leaving
// only the few FP64 additions that touch the FP64 state. Everything here is plain C++
// (host and device), so the CPU tests check it bit for bit against the host's own casts.
#pragma once
#include <cstdint>
#include <cmath>
#include <cstring>

#ifdef __CUDACC__
#define ATHG_HD __host__ __device__ __forceinline__
#else
#define ATHG_HD inline
#endif

namespace athg {

ATHG_HD uint32_t bits_f(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
ATHG_HD uint64_t bits_d(double d) { uint64_t u; std::memcpy(&u, &d, 8); return u; }
ATHG_HD float from_bits_f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
ATHG_HD double from_bits_d(uint64_t u) { double d; std::memcpy(&d, &u, 8); return d; }

// binary32 -> binary64, exact for normal numbers; zero and subnormal inputs give a
// signed zero (the FP32 kernels flush subnormals), infinities and NaNs keep their class.
ATHG_HD double f2d_int(float f) {
  const uint32_t x = bits_f(f);
  const uint32_t a = x & 0x7fffffffu;
  const uint64_t s = (uint64_t)(x & 0x80000000u) << 32;
  uint64_t m = ((uint64_t)a << 29) + 0x3800000000000000ull;  // exponent bias 127 -> 1023
  if (a < 0x00800000u) m = 0ull;
  if (a >= 0x7f800000u) m = 0x7ff0000000000000ull | ((uint64_t)(a & 0x007fffffu) << 29);
  return from_bits_d(s | m);
}

// binary64 -> binary32 rounded to nearest, ties to even; results that round below the
// smallest normal binary32 flush to a signed zero, results above the largest become
// infinity. Works on the two 32-bit halves: masking the sign off the whole 64-bit
// pattern is the idiom compilers turn back into an FP64 absolute value.
ATHG_HD float d2f_int(double d) {
  const uint64_t x = bits_d(d);
  const uint32_t hi = (uint32_t)(x >> 32), lo = (uint32_t)x;
  const uint32_t s = hi & 0x80000000u;
  const uint32_t ed = (hi >> 20) & 0x7ffu;                  // binary64 exponent
  const uint32_t m23 = ((hi & 0x000fffffu) << 3) | (lo >> 29);  // kept mantissa bits
  const uint32_t rb = lo & 0x1fffffffu;                      // the 29 dropped bits
  const uint32_t up = (rb > 0x10000000u || (rb == 0x10000000u && (m23 & 1u))) ? 1u : 0u;
  const int fe = (int)ed - 896;                              // binary32 exponent
  uint32_t m;
  if (ed == 0x7ffu) m = (m23 | (hi & 0x000fffffu) | lo) ? 0x7fc00000u : 0x7f800000u;
  else if (fe >= 255) m = 0x7f800000u;
  else if (fe <= 0) m = (fe == 0 && m23 == 0x7fffffu && up) ? 0x00800000u : 0u;
  else m = (((uint32_t)fe << 23) | m23) + up;               // a carry moves into the exponent
  return from_bits_f(s | m);
}

// Knuth's TwoSum: s + e == a + b exactly in round-to-nearest binary32 arithmetic (only
// additions, so no contraction into FMA can change it)
ATHG_HD void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// (a - b) + (c - d) + (f - h) as an unevaluated pair hi + lo (cascaded TwoSum,
// Ogita-Rump-Oishi Sum2): |hi + lo - exact| <= about 2^-44 (|a|+|b|+...+|h|)
ATHG_HD void sum3diff(float a, float b, float c, float d, float f, float h, float& hi,
                      float& lo) {
  float s1, e1, s2, e2, s3, e3, t, e4, e5;
  two_sum(a, -b, s1, e1);
  two_sum(c, -d, s2, e2);
  two_sum(f, -h, s3, e3);
  two_sum(s1, s2, t, e4);
  two_sum(t, s3, hi, e5);
  lo = ((e1 + e2) + e3) + (e4 + e5);
}

// (a - b) + (c - d) as hi + lo: |hi + lo - exact| <= about 2^-45 (|a|+|b|+|c|+|d|)
ATHG_HD void sum2diff(float a, float b, float c, float d, float& hi, float& lo) {
  float s1, e1, s2, e2, e3;
  two_sum(a, -b, s1, e1);
  two_sum(c, -d, s2, e2);
  two_sum(s1, s2, hi, e3);
  lo = (e1 + e2) + e3;
}

// ---- double-float (unevaluated FP32 pairs hi + lo) --------------------------------------
// Used where an FP64-class result is needed from FP64 inputs without FP64 instructions:
// |hi + lo - x| <= about 2^-46 |x|.
struct ff {
  float hi, lo;
};

// Split binary64 x into hi = x rounded to binary32 and lo ~ x - hi, on the integer pipe:
// the 29 mantissa bits that rounding drops become a signed integer r, |r| <= 2^28, kept
// to 22 bits and scaled by the exponent. |x| outside [2^-80, 2^120]: lo = 0.
// split_ff_general handles every input; split_ff below takes a short path for the usual
// range and gives the same bits.
ATHG_HD ff split_ff_general(double x) {
  // the rounding of d2f_int, and its remainder, on the 32-bit halves
  const uint64_t b = bits_d(x);
  const uint32_t hi32 = (uint32_t)(b >> 32), lo32 = (uint32_t)b;
  const uint32_t s = hi32 & 0x80000000u;
  const uint32_t ed = (hi32 >> 20) & 0x7ffu;
  const uint32_t m23 = ((hi32 & 0x000fffffu) << 3) | (lo32 >> 29);
  const uint32_t rb = lo32 & 0x1fffffffu;
  const uint32_t up = (rb > 0x10000000u || (rb == 0x10000000u && (m23 & 1u))) ? 1u : 0u;
  const int fe = (int)ed - 896;
  uint32_t m;
  if (ed == 0x7ffu) m = (m23 | (hi32 & 0x000fffffu) | lo32) ? 0x7fc00000u : 0x7f800000u;
  else if (fe >= 255) m = 0x7f800000u;
  else if (fe <= 0) m = (fe == 0 && m23 == 0x7fffffu && up) ? 0x00800000u : 0u;
  else m = (((uint32_t)fe << 23) | m23) + up;
  ff o;
  o.hi = from_bits_f(s | m);
  // remainder x - hi in units of 2^(e-1075): the dropped bits, less 2^29 when rounded up
  const int32_t r = (int32_t)rb - (int32_t)(up << 29);  // |r| <= 2^28
  // (r >> 6) as a float through the 1.5 * 2^23 offset (exact for |r >> 6| <= 2^22), times
  // 2^(e - 1075 + 6); |x| outside [2^-80, 2^120]: lo = 0
  const float q = from_bits_f(0x4b400000u + (uint32_t)(r >> 6)) - 12582912.0f;
  const int se = (int)ed - 1069 + 127;
  const bool ok = se > 0 && se < 255 && ed >= 943u && ed <= 1143u;
  const float scale = from_bits_f((uint32_t)(ok ? se : 1) << 23);
  const float lo = ok ? q * scale : 0.0f;
  o.lo = s ? -lo : lo;
  return o;
}

ATHG_HD ff split_ff(double x) {
  const uint64_t b = bits_d(x);
  const uint32_t hi32 = (uint32_t)(b >> 32), lo32 = (uint32_t)b;
  const uint32_t a = hi32 & 0x7fffffffu;
  // 2^-80 <= |x| < 2^120 (binary64 exponent 943..1142): hi is a normal binary32 whatever
  // the rounding, and the remainder's scale is a normal binary32 too
  if (a - 0x3af00000u >= 0x0c800000u) return split_ff_general(x);
  // exponent rebiased and the 23 kept mantissa bits, in one word
  const uint32_t m = ((a - 0x38000000u) << 3) | (lo32 >> 29);
  const uint32_t rb = lo32 & 0x1fffffffu;
  const uint32_t up = (rb > 0x10000000u || (rb == 0x10000000u && (m & 1u))) ? 1u : 0u;
  const uint32_t s = hi32 & 0x80000000u;
  ff o;
  o.hi = from_bits_f(s | (m + up));
  const int32_t r = (int32_t)rb - (int32_t)(up << 29);
  const float q = from_bits_f(0x4b400000u + (uint32_t)(r >> 6)) - 12582912.0f;
  const float lo = q * from_bits_f(((a >> 20) - 942u) << 23);
  o.lo = s ? -lo : lo;
  return o;
}

// error-free product of two binary32 numbers (needs a fused multiply-add)
ATHG_HD void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = std::fma(a, b, -p);
}

ATHG_HD ff ff_renorm(float s, float e) {
  ff o;
  two_sum(s, e, o.hi, o.lo);
  return o;
}

ATHG_HD ff ff_add(ff a, ff b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  return ff_renorm(s, e);
}

ATHG_HD ff ff_sub(ff a, ff b) {
  ff nb;
  nb.hi = -b.hi;
  nb.lo = -b.lo;
  return ff_add(a, nb);
}

ATHG_HD ff ff_mul(ff a, ff b) {
  float p, e;
  two_prod(a.hi, b.hi, p, e);
  e = std::fma(a.hi, b.lo, e);
  e = std::fma(a.lo, b.hi, e);
  return ff_renorm(p, e);
}

ATHG_HD ff ff_sqr(ff a) {
  float p, e;
  two_prod(a.hi, a.hi, p, e);
  e = std::fma(2.0f * a.hi, a.lo, e);
  return ff_renorm(p, e);
}

ATHG_HD ff ff_scale(ff a, float pow2) {  // exact for a power of two
  ff o;
  o.hi = a.hi * pow2;
  o.lo = a.lo * pow2;
  return o;
}

// 1 / a from an FP32 reciprocal and one double-float Newton step
ATHG_HD ff ff_recip(ff a) {
  const float r = 1.0f / a.hi;
  // residual 1 - a r in double-float, then r + r (1 - a r)
  float p, e;
  two_prod(a.hi, r, p, e);
  const float res = ((1.0f - p) - e) - a.lo * r;
  return ff_renorm(r, r * res);
}

// value rounded to binary32
ATHG_HD float ff_f(ff a) { return a.hi + a.lo; }

// a > b for double-float values (normalised: |lo| <= ulp(hi) / 2)
ATHG_HD bool ff_gt(ff a, ff b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }

// 6 c - (n[0] + ... + n[5]) of seven binary64 values, as a double-float pair, without FP64
// instructions. Each value becomes a 64-bit integer in units of 2^(emax - 1081), emax the
// largest of the seven binary64 exponents, so the largest mantissa sits below bit 59; a
// value loses only the bits below that unit (at most 2^-58 of the largest |value|). The
// seven-point sum is then exact in the integer (|sum| < 1.5 * 2^62) and is rounded once
// into hi + lo (|error| <= about 2^-47 |sum|), where FP64 would round after each of six
// operations. Returns false, with out untouched, for values that are not finite or whose
// scale falls outside [2^-126, 2^64] (|c| and |n| roughly outside [2^-68, 2^122]); the
// caller then takes FP64.
ATHG_HD bool lap7_ff(double c, const double* n, ff& out) {
  uint64_t b[7];
  b[0] = bits_d(c);
  for (int q = 0; q < 6; ++q) b[q + 1] = bits_d(n[q]);
  int ex[7];
  int emax = 1;
  for (int q = 0; q < 7; ++q) {
    const int e = (int)((b[q] >> 52) & 0x7ffu);
    ex[q] = e ? e : 1;  // subnormals: the exponent of the smallest normals
    emax = ex[q] > emax ? ex[q] : emax;
  }
  if (emax < 955 || emax > 1145) return false;  // also excludes infinities and NaNs
  int64_t x[7];
  for (int q = 0; q < 7; ++q) {
    const uint64_t mant = (b[q] & 0x000fffffffffffffull) |
                          (((b[q] >> 52) & 0x7ffu) ? 0x0010000000000000ull : 0ull);
    const int sh = emax - ex[q];
    const uint64_t m = sh < 64 ? ((mant << 6) >> sh) : 0ull;
    x[q] = (b[q] >> 63) ? -(int64_t)m : (int64_t)m;
  }
  const int64_t sum = 6 * x[0] - (((x[1] + x[2]) + (x[3] + x[4])) + (x[5] + x[6]));
  const float hi = (float)sum;                        // rounded to nearest
  const float lo = (float)(sum - (int64_t)hi);        // the remainder, |.| <= 2^38
  const float scale = from_bits_f((uint32_t)(emax - 1081 + 127) << 23);
  out.hi = hi * scale;
  out.lo = lo * scale;
  return true;
}

// Division by an invariant d (1 <= d < 2^31) for numerators 0 <= a < 2^31 with the high
// half of one 32 x 32-bit product and a shift (Granlund and Montgomery's round-up method):
// with l = ceil(log2 d) and m = ceil(2^(31 + l) / d) < 2^32,
// a m / 2^(31 + l) = a / d + a r / (d 2^(31 + l)) with 0 <= r < d, and the second term is
// below 2^-l <= 1 / d, so it never reaches the next integer: floor(a m / 2^(31 + l)) =
// floor(a / d). As 2a < 2^32, that quotient is the high word of (2a) m shifted by l.
struct FastDiv {
  uint32_t mul;
  uint32_t shift;  // l
};
inline FastDiv fastdiv_make(uint32_t d) {
  uint32_t l = 0;
  while ((1ull << l) < d) ++l;
  const uint64_t m = ((1ull << (31 + l)) + d - 1) / d;
  return FastDiv{(uint32_t)m, l};
}
ATHG_HD int fastdiv(int a, FastDiv f) {
  const uint32_t a2 = (uint32_t)a << 1;
#ifdef __CUDA_ARCH__
  const uint32_t hi = __umulhi(a2, f.mul);
#else
  const uint32_t hi = (uint32_t)(((uint64_t)a2 * f.mul) >> 32);
#endif
  return (int)(hi >> f.shift);
}

// Quotient a / b for 0 <= a < 2^12 and 1 <= b <= 2^10, given rb = 1 / b rounded to binary32:
// one FP32 multiply in place of an integer division. (a + 0.5) / b lies at least 0.5 / b
// from every integer, and the two roundings move (a + 0.5) * rb by at most about
// 2^-23 (a + 0.5) / b, below 2^-12 / b, so truncation gives the exact quotient.
ATHG_HD int div_small(int a, float rb) { return (int)(((float)a + 0.5f) * rb); }

}  // namespace athg
