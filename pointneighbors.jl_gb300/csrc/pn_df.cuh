// pn_df.cuh -- double-float arithmetic: a value is the unevaluated sum hi + lo of two
// Float32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits.  GB300's Float64
// units run at a small fraction of its Float32 rate, so the Float64 pair functions' sums
// (WCSPH density and force) are formed in this arithmetic on the Float32 units, within
// about 2^-44 of the exact values, far inside the 1e-12 relative tolerance of the Float64
// results.
//
// The building blocks are the classical error-free transformations:
//   two_sum (Knuth): s = fl(a + b) and the exact error e, a + b = s + e;
//   two_prod (with a fused multiply-add): p = fl(a b), e = fma(a, b, -p), a b = p + e;
// and the double-length operations built on them (Dekker 1971; Hida, Li and Bailey's
// double-double algorithms), with one correction step for quotient and square root.  Every
// operation is an explicitly rounded intrinsic so that the compiler cannot contract or
// reassociate a step the error analysis relies on.
#pragma once

#include <cuda_runtime.h>

namespace pn {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float hi, float lo = 0.0f) { return df{hi, lo}; }

// a + b = s + e exactly (any a, b)
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df{s, e};
}
// the same when |a| >= |b| (or a = 0)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
// a b = p + e exactly (barring underflow)
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }

// a + b: both error terms carried (the accurate sum)
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
// a + b for a, b >= 0 (d^2, the density sum): nothing cancels, so the low parts need no
// error term of their own
__device__ __forceinline__ df df_add_pos(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, p.lo);
  p.lo = __fmaf_rn(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_sqr(df a) {
  df p = two_prod(a.hi, a.hi);
  p.lo = __fmaf_rn(__fmul_rn(2.0f, a.hi), a.lo, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
// a / b (0 < |b| < 2^126): the Float32 quotient q1, the remainder a - q1 b in
// double-float (exact for any q1), a second quotient and remainder, a last correction.  The
// remainders are exact, so the Float32 quotients need not be correctly rounded: each
// approximate quotient (a few ulp) only enlarges the next, smaller correction.
__device__ __forceinline__ df df_div(df a, df b) {
  const float q1 = __fdividef(a.hi, b.hi);
  const df r = df_sub(a, df_mul_f(b, q1));
  const float q2 = __fdividef(r.hi, b.hi);
  df q = fast_two_sum(q1, q2);
  const df r2 = df_sub(r, df_mul_f(b, q2));
  return df_add_f(q, __fdividef(r2.hi, b.hi));
}
// sqrt(a), a >= 0: s = sqrt(a.hi) correctly rounded, then s + (a - s^2) / (2 s) (one Newton
// step; the correction is 2^-24 of s, so its own few-ulp quotient error is 2^-46 of s)
__device__ __forceinline__ df df_sqrt(df a) {
  if (!(a.hi > 0.0f)) return df{0.0f, 0.0f};
  const float s = __fsqrt_rn(a.hi);
  const df e = df_sub(a, two_prod(s, s));
  return fast_two_sum(s, __fdividef(e.hi, __fmul_rn(2.0f, s)));
}
__device__ __forceinline__ bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool df_gt(df a, df b) { return df_lt(b, a); }

// Float64 <-> double-float (each direction one Float64 operation and two conversions; used
// per point, not per pair)
__host__ __device__ __forceinline__ df df_from(double x) {
  const float hi = (float)x;
  return df{hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

// The exact difference (xa + xb + xc) - (ya + yb + yc) of two Float64 values given as their
// three-part Float32 splits (x = xa + xb + xc exactly, each part the Float32 rounding of
// what the previous parts leave), to double-float precision: the two leading parts'
// differences are taken exactly (two_sum) and summed exactly into hi + e; the remaining
// terms (the two sums' errors, the third parts' difference and e) are each below an ulp of
// the leading parts and are added in Float32, then renormalised -- within 2^-46 of the
// difference (tests/test_df_arith.py checks this against exact rationals).
__device__ __forceinline__ df df_diff3(float xa, float xb, float xc, float ya, float yb,
                                       float yc) {
  const df a = two_sum(xa, -ya);
  const df b = two_sum(xb, -yb);
  const df s = two_sum(a.hi, b.hi);
  const float low =
      __fadd_rn(__fadd_rn(__fadd_rn(a.lo, b.lo), __fsub_rn(xc, yc)), s.lo);
  return fast_two_sum(s.hi, low);
}

}  // namespace pn
