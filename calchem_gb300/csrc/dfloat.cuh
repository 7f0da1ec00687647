// dfloat.cuh -- double-float ("float-float") arithmetic on the FP32 pipe.
//
// A value is an unevaluated sum hi + lo of two floats with |lo| <= ulp(hi) / 2, giving ~48
// significant bits.  The building blocks are the classical error-free transformations (Knuth's
// TwoSum, Dekker's Fast2Sum, and the FMA-based TwoProd), as published in e.g. Muller et al.,
// "Handbook of Floating-Point Arithmetic".  All additions and multiplications inside the
// transformations use the explicit round-to-nearest intrinsics so the compiler cannot contract or
// reassociate them.  GB300 runs FP32 at ~64x its FP64 rate, so ~10-20 FP32 operations per
// double-float operation are far cheaper than native FP64.
#pragma once

#include <cuda_runtime.h>

namespace cxc {

struct df32 {
  float hi, lo;
};

__device__ __forceinline__ df32 df_make(float hi, float lo) { return df32{hi, lo}; }

__device__ __forceinline__ df32 df_from_double(double x) {
  const float hi = __double2float_rn(x);
  return df32{hi, __double2float_rn(x - (double)hi)};
}

__device__ __forceinline__ double df_to_double(df32 a) { return (double)a.hi + (double)a.lo; }

// TwoSum: s + e == a + b exactly.
__device__ __forceinline__ df32 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df32{s, e};
}

// Fast2Sum (|a| >= |b|): s + e == a + b exactly.
__device__ __forceinline__ df32 fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df32{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// TwoProd with FMA: p + e == a * b exactly.
__device__ __forceinline__ df32 two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df32{p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  df32 s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df32 df_add_f(df32 a, float b) {
  df32 s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df32 df_neg(df32 a) { return df32{-a.hi, -a.lo}; }

__device__ __forceinline__ df32 df_sub(df32 a, df32 b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
  df32 p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ df32 df_mul_f(df32 a, float b) {
  df32 p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

// a / b for 2^-126 < |b| < 2^126: an approximate FP32 quotient (a few ulp) and one correction from
// the exact remainder (Dekker); the correction's own error is ~1e-7 of a term ~1e-7 of the result.
__device__ __forceinline__ df32 df_div(df32 a, df32 b) {
  const float q1 = __fdividef(a.hi, b.hi);
  const df32 p = two_prod(q1, b.hi);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p.hi), p.lo), __fsub_rn(a.lo, __fmul_rn(q1, b.lo)));
  return two_sum(q1, __fdividef(r, b.hi));
}

// sqrt(a) for a >= 0: the FP32 root and one Newton correction from the exact residual a - s^2
// (Karp and Markstein's form of the correction).
__device__ __forceinline__ df32 df_sqrt(df32 a) {
  if (!(a.hi > 0.f)) return df32{0.f, 0.f};
  const float s0 = sqrtf(a.hi);
  const df32 p = two_prod(s0, s0);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p.hi), p.lo), a.lo);
  return two_sum(s0, __fdividef(r, __fmul_rn(2.f, s0)));
}

// Exact scaling by a power of two (as long as no underflow/overflow occurs).
__device__ __forceinline__ df32 df_ldexp(df32 a, int e) { return df32{ldexpf(a.hi, e), ldexpf(a.lo, e)}; }

// 2^k as a float: exact for -149 <= k <= 127 (a normal number for k >= -126).  x * pow2f(k) is then
// x 2^k rounded once, as ldexpf(x, k) gives it.
__device__ __forceinline__ float pow2f(int k) {
  return (k >= -126 && k <= 127) ? __int_as_float((k + 127) << 23) : ldexpf(1.f, k);
}

// exp(-x) for x >= 0 given as a double-float, relative error ~1e-13 (before underflow).
// Method: x = (64 k + j) ln2/64 + r with |r| <= ln2/128 (Cody-Waite reduction with ln2/64 split
// into a 10-bit head, so n * head is exact, and two tails), exp(-r) from its Taylor series to
// r^4 (truncation < r^5/120 ~ 4e-14), times a table of 2^(-j/64) held as double-floats, times
// 2^-k.  tab points at 64 double-float entries of 2^(-j/64).
__device__ __forceinline__ df32 df_exp_neg(df32 x, const df32* tab) {
  if (!(x.hi < 100.f)) return df32{0.f, 0.f};  // below FP32's range for our purposes
  const float n = rintf(x.hi * 92.33248261689366f);            // 64 / ln2
  const float L1 = 0.010833740234375f, L2 = -3.3155381515825866e-06f, L3 = 2.5727683872212026e-14f;
  // r = x - n * (L1 + L2 + L3): n * L1 exact; the rest carried as a double-float
  const float t1 = __fsub_rn(x.hi, __fmul_rn(n, L1));
  df32 r = two_sum(t1, x.lo);
  r = df_add(r, df_neg(two_prod(n, L2)));
  r = df_add_f(r, -__fmul_rn(n, L3));
  // exp(-r) = 1 - r + r^2/2 - r^3/6 + r^4/24, the small terms in FP32 (|q| < 2e-5)
  const float rh = r.hi;
  const float q = rh * rh * (0.5f + rh * (-1.f / 6.f + rh * (1.f / 24.f)));
  df32 e = df_add(df32{1.f, 0.f}, df_neg(r));
  e = df_add_f(e, q);
  const int ni = (int)n;
  const int j = ni & 63;
  const int k = ni >> 6;  // n = 64 k + j, j in [0, 64)
  return df_ldexp(df_mul(tab[j], e), -k);
}

}  // namespace cxc
