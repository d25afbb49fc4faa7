// Double-float arithmetic on the FP32 pipe: a value is an unevaluated sum
// hi + lo of two floats (Dekker, "A floating-point technique for extending
// the available precision", Numer. Math. 18, 1971; Knuth, TAOCP vol. 2,
// 4.2.2). GB300 issues FP32 at 58 times its FP64 rate, so a stencil row in
// double-float (about 48 significant bits) costs less than the same row in
// FP64 where FP64 throughput is the bound. Every step below is an
// error-free transformation or a documented rounding; nothing relies on
// reassociation.
#pragma once

#include <cstdint>

namespace ibm {

// s + e == a + b exactly (Knuth's two-sum).
__device__ __forceinline__ void df_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// s + e == a + b exactly when |a| >= |b| or a == 0 (Dekker's fast two-sum).
__device__ __forceinline__ void df_fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

// (hi, lo) += (ch + cl) * (xh + xl): the leading product exactly (fma
// residual), the cross terms rounded in FP32, cl * xl (2^-48 of the product)
// dropped; then a double-float addition.
__device__ __forceinline__ void df_fma(float &hi, float &lo, float ch, float cl, float xh, float xl) {
  const float p = __fmul_rn(ch, xh);
  float pe = __fmaf_rn(ch, xh, -p);
  pe = __fmaf_rn(ch, xl, __fmaf_rn(cl, xh, pe));
  float s, e;
  df_two_sum(hi, p, s, e);
  e = __fadd_rn(e, __fadd_rn(lo, pe));
  df_fast_two_sum(s, e, hi, lo);
}

// (rh, rl) = (ah, al) - (bh, bl).
__device__ __forceinline__ void df_sub(float ah, float al, float bh, float bl, float &rh, float &rl) {
  float s, e;
  df_two_sum(ah, -bh, s, e);
  e = __fadd_rn(e, __fsub_rn(al, bl));
  df_fast_two_sum(s, e, rh, rl);
}

// v == hi + lo to within 2^-48 |v|, from the bits of v (integer operations
// only; no FP64 instruction): hi holds the leading 24 significand bits
// (truncated, so v - hi is exact in FP64), lo the next 29 rounded to a float.
// |v| below 2^-126 is flushed to zero, lo is flushed when its weight falls
// below 2^-126 (|v| below 2^-74), |v| at or above 2^128 gives an infinity,
// NaN stays NaN.
__device__ __forceinline__ void df_split(double v, float &hi, float &lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned sgn = (unsigned)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7ff);
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  if (e == 0x7ff) {  // infinity or NaN
    hi = __uint_as_float(sgn | 0x7f800000u | (m ? 0x00400000u : 0u));
    lo = 0.0f;
    return;
  }
  const int fe = e - 1023 + 127;  // float biased exponent of the leading bit
  if (fe <= 0) { hi = __uint_as_float(sgn); lo = 0.0f; return; }
  if (fe >= 255) { hi = __uint_as_float(sgn | 0x7f800000u); lo = 0.0f; return; }
  hi = __uint_as_float(sgn | ((unsigned)fe << 23) | (unsigned)(m >> 29));
  const unsigned L = (unsigned)(m & 0x1FFFFFFFull);  // weight 2^(e - 1075)
  const int le = e - 1075 + 127;
  if (le <= 0 || L == 0) { lo = 0.0f; return; }
  const float l = __fmul_rn(__uint2float_rn(L), __uint_as_float((unsigned)le << 23));
  lo = sgn ? -l : l;
}

}  // namespace ibm
