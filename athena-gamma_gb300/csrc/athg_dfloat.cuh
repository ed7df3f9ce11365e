// athg_dfloat.cuh -- double-float numbers for the reconstruction and Riemann solvers of the
// double-float flux path (precision ATHG_DFLOAT).
//
// A value is the unevaluated sum hi + lo of two binary32 numbers with |lo| <= ulp(hi)/2:
// about 48 significant bits from FP32-pipe instructions only (FP64 instructions issue at
// 1/64 of the FP32 rate on this GPU). The operations follow the classic double-float
// algorithms (Dekker 1971; Hida, Li and Bailey, "Library for double-double and quad-double
// arithmetic", 2000): error-free TwoSum / TwoProduct of the high parts, the low parts added
// in, and a renormalisation; division and square root take one correction step from the
// FP32 estimate. Relative error of one operation is about 2^-44 or better, absolute error
// in a cancellation about 2^-48 of the operands, the behaviour of FP64 to within a factor
// of 2^5. Comparisons order normalised pairs exactly.
//
// The stage templates (athg_device.cuh) take the type as T: literals such as T(0.5) are
// folded at compile time; runtime doubles enter through df_of (an exact split on the
// integer pipe) and leave through dbl (hi + lo widened and added).
#pragma once
#include "athg_numeric.h"

namespace athg {

struct dfl {
  float hi, lo;
  dfl() = default;
  __host__ __device__ constexpr dfl(float h, float l) : hi(h), lo(l) {}
  // compile-time constants (and rare runtime doubles: the FP64 conversions are then real)
  __host__ __device__ constexpr dfl(double x)
      : hi((float)x), lo((float)(x - (double)(float)x)) {}
};

// exact split of an FP64 value (integer pipe; see split_ff)
__device__ __forceinline__ dfl df_of(double x) {
  const ff s = split_ff(x);
  return dfl(s.hi, s.lo);
}
// the FP64 value nearest hi + lo
__device__ __forceinline__ double dbl(dfl a) { return f2d_int(a.hi) + f2d_int(a.lo); }

__device__ __forceinline__ dfl df_fast(float s, float e) {  // |s| >= |e| expected
  const float h = s + e;
  return dfl(h, e - (h - s));
}

__device__ __forceinline__ dfl operator+(dfl a, dfl b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  return df_fast(s, e);
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.hi, -a.lo); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return df_fast(p, e);
}
__device__ __forceinline__ dfl operator/(dfl a, dfl b) {
  const float q1 = a.hi * __frcp_rn(b.hi);
  // remainder a - q1 b, then one correction
  const float p = b.hi * q1;
  const float pe = fmaf(b.hi, q1, -p);
  const float r = (((a.hi - p) - pe) + a.lo) - q1 * b.lo;
  const float q2 = r * __frcp_rn(b.hi);
  return df_fast(q1, q2);
}
__device__ __forceinline__ dfl sqrt(dfl a) {
  if (!(a.hi > 0.0f)) return dfl(a.hi == 0.0f ? 0.0f : __fsqrt_rn(a.hi), 0.0f);
  const float s = __fsqrt_rn(a.hi);
  const float p = s * s;
  const float pe = fmaf(s, s, -p);
  const float r = ((a.hi - p) - pe) + a.lo;
  return df_fast(s, r * (0.5f * __frcp_rn(s)));
}
__device__ __forceinline__ dfl fabs(dfl a) { return a.hi < 0.0f ? -a : a; }

__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b) { a = a + b; return a; }
__device__ __forceinline__ dfl& operator-=(dfl& a, dfl b) { a = a - b; return a; }
__device__ __forceinline__ dfl& operator*=(dfl& a, dfl b) { a = a * b; return a; }

__device__ __forceinline__ bool operator<(dfl a, dfl b) {
  return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo);
}
__device__ __forceinline__ bool operator>(dfl a, dfl b) { return b < a; }
__device__ __forceinline__ bool operator<=(dfl a, dfl b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dfl a, dfl b) { return !(a < b); }
__device__ __forceinline__ bool operator==(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(dfl a, dfl b) { return !(a == b); }

// the stage templates' comparison helpers (athg_device.cuh) for double-float operands
__device__ __forceinline__ bool lt(dfl a, dfl b) { return a < b; }
__device__ __forceinline__ bool le(dfl a, dfl b) { return a <= b; }
__device__ __forceinline__ bool gt(dfl a, dfl b) { return b < a; }
__device__ __forceinline__ bool ge(dfl a, dfl b) { return b <= a; }
__device__ __forceinline__ dfl fab(dfl x) { return fabs(x); }

}  // namespace athg
