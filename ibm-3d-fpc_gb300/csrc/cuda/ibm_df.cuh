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

// (hi, lo) += (ch + cl) * x for a float x: ch * x exactly (fma residual),
// cl * x rounded in FP32 (2^-48 of the product); then a double-float addition.
__device__ __forceinline__ void df_fma1(float &hi, float &lo, float ch, float cl, float x) {
  const float p = __fmul_rn(ch, x);
  const float pe = __fmaf_rn(cl, x, __fmaf_rn(ch, x, -p));
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

// v == hi + lo to within 2^-46 |v| from the bits of v, on the integer and
// FP32 pipes without a conversion instruction: hi holds the leading 24
// significand bits (truncated), lo the next 23 (truncated). For a biased
// exponent e in (896, 1151) one funnel shift brings the low 8 exponent bits
// and 23 fraction bits into place and flipping bit 30 rebiases the exponent
// (e - 896 == (e mod 256) xor 128 there); lo is (2^23 + L) 2^-46 - 2^-23,
// exact in one FMA, times hi's signed power of two. |v| below 2^-126 gives
// a signed zero, lo underflows gradually below 2^-81 (an absolute error under
// 2^-104); |v| at or above 2^128, infinities and NaN take df_split.
__device__ __forceinline__ void df_split_fast(double v, float &hi, float &lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(v);
  const unsigned uh = (unsigned)(u >> 32), ul = (unsigned)u;
  const unsigned e = (uh >> 20) & 0x7FFu;
  if (e >= 1151u) { df_split(v, hi, lo); return; }
  const unsigned sgn = uh & 0x80000000u;
  const unsigned hb = ((__funnelshift_l(ul, uh, 3) ^ 0x40000000u) & 0x7FFFFFFFu) | sgn;
  const float raw = __uint_as_float(0x4B000000u | ((ul >> 6) & 0x7FFFFFu));
  const float lf = __fmaf_rn(raw, 1.4210854715202004e-14f, -1.1920928955078125e-07f);  // L 2^-46
  const float lm = __fmul_rn(lf, __uint_as_float(hb & 0xFF800000u));
  const bool tiny = e <= 896u;
  hi = __uint_as_float(tiny ? sgn : hb);
  lo = tiny ? 0.0f : lm;
}

// A double-float value and the operations the dense kernels need. Sums and
// products carry about 2^-47 of their operands' size.
struct DF {
  float h, l;
};
__device__ __forceinline__ DF df_of(double v) {
  DF r;
  df_split_fast(v, r.h, r.l);
  return r;
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s, e;
  df_two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  DF r;
  df_fast_two_sum(s, e, r.h, r.l);
  return r;
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.h, -a.l}; }
__device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, e));
  DF r;
  df_fast_two_sum(p, e, r.h, r.l);
  return r;
}
// times an exact power of two (no rounding unless the result leaves the
// normal range)
__device__ __forceinline__ DF df_scale(DF a, float p2) { return DF{__fmul_rn(a.h, p2), __fmul_rn(a.l, p2)}; }
// widened to FP64: two exact conversions and one rounding add
__device__ __forceinline__ double df_to_double(DF a) { return __dadd_rn((double)a.h, (double)a.l); }

}  // namespace ibm
