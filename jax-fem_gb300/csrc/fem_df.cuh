// Double-float arithmetic on the FP32 pipes: a value is an unevaluated float pair h + l with
// |l| <= ulp(h)/2 (~48-bit mantissa), built with error-free transformations (two-sum, and
// two-product through fmaf).  GB300's FP64 pipe runs at ~1/64 of its FP32 rate, so the mixed
// solver's SpMV and vectors and the double-float assembly kernels use these instead of FP64.
// Also the DF48 matrix format's decode (FP32 hi + int16 correction scaled to the ulp of hi) and
// bit-level FP32 / FP64 conversions that avoid the FP64 pipe.
#pragma once

#include <stdint.h>

namespace fem {

__device__ __forceinline__ float df_lo_scale(float hi) {
  const int e = (__float_as_int(hi) >> 23) & 0xFF;
  return e > 39 ? __int_as_float((e - 39) << 23) : 0.0f;   // 2^(e - 166) = ulp(hi) / 2^16
}

// DF48 correction without an int->float conversion: base is the float 1.5 * 2^(E-143) (E the
// exponent field of hi); adding q (|q| < 2^15) to its mantissa field gives (1.5 + q/2^23) *
// 2^(E-143), and subtracting base leaves exactly q * 2^(E-166) = q * ulp(hi) / 2^16.  Encoders
// write q = 0 whenever E <= 39, where base may wrap: the result is then 0 as required.
__device__ __forceinline__ float df48_lo(float hi, int q) {
  const int base = (__float_as_int(hi) & 0x7f800000) + (0x400000 - (16 << 23));
  return __int_as_float(base + q) - __int_as_float(base);
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& err) {
  s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
}

// A df value is an unevaluated float pair h + l with |l| <= ulp(h)/2 (~48-bit mantissa).
// GB300's FP64 pipe is ~1/64 of its FP32 rate, so the mixed solver keeps x, r, p, q in this
// form and touches FP64 only to finish per-thread dot partials and in the scalar recurrences.
struct df2 { float h, l; };

__device__ __forceinline__ df2 df_fast(float s, float e) {  // |s| >= |e|
  const float h = s + e;
  return df2{h, e - (h - s)};
}
__device__ __forceinline__ df2 df_add(df2 a, df2 b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e += a.l + b.l;
  return df_fast(s, e);
}
__device__ __forceinline__ df2 df_mul(df2 a, df2 b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_fast(p, e);
}
__device__ __forceinline__ df2 df_of(double d) {
  const float h = __double2float_rn(d);
  return df2{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double df_dbl(df2 a) { return (double)a.h + (double)a.l; }

// An FP64 value as a double-float pair built from its bits with integer and FP32 operations only
// (GB300's FP64 pipe runs ~1/64 of the FP32 rate): h keeps the sign, the exponent and the leading
// 24 significand bits, l the next 29 bits (rounded to 24), renormalised.  For |v| inside FP32's
// normal range; the CG's vectors are range-scaled to an RMS near 1.  Values whose l would fall
// below FP32's normal range keep h only (|v| below ~2^-74: far under the vectors' rounding).
__device__ __forceinline__ df2 df_from_bits(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const int e = (int)((hw >> 20) & 0x7FFu) - 1023;          // unbiased exponent
  const unsigned sgn = hw & 0x80000000u;
  if (e < -126) return df2{0.f, 0.f};
  if (e > 127) return df2{__int_as_float(sgn | 0x7F800000u), 0.f};
  const float h = __int_as_float(sgn | ((unsigned)(e + 127) << 23) | ((hw & 0xFFFFFu) << 3) | (lw >> 29));
  float l = 0.f;
  if (e - 52 >= -126) l = __int_as_float(sgn | 0x3F800000u) * (float)(lw & 0x1FFFFFFFu) *
                          __int_as_float((unsigned)(e - 52 + 127) << 23);
  return df_fast(h, l);
}

// accumulate a*b into (sh, sl) without renormalising every step
__device__ __forceinline__ void df_acc(float& sh, float& sl, df2 a, df2 b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  float t, te;
  two_sum(sh, p, t, te);
  sl += te + e;
  sh = t;
}

// Two independent df_acc at once on Blackwell's paired FP32 instructions (FMUL2 / FFMA2 / FADD2,
// sm_100+): component k of (sh, sl) accumulates ah.k * (xh.k + xl.k) + al.k * xh.k exactly as
// df_acc does -- every paired operation rounds per component like its scalar form, and the
// subtractions of the two-sum are FFMA2 with a -1 multiplier (exact).  nxh = -xh (negated once
// per gathered x, reused across a block's rows) gives -p without a separate negation.
__device__ __forceinline__ void df_acc2(float2& sh, float2& sl, float2 ah, float2 al, float2 xh, float2 nxh,
                                        float2 xl) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 np = __fmul2_rn(ah, nxh);        // -p, p = fl(ah xh)
  float2 e = __ffma2_rn(ah, xh, np);             // ah xh - p, exact
  e = __ffma2_rn(ah, xl, e);
  e = __ffma2_rn(al, xh, e);
  const float2 t = __ffma2_rn(np, m1, sh);       // fl(sh + p)
  const float2 bb = __ffma2_rn(sh, m1, t);       // fl(t - sh)
  const float2 tb = __ffma2_rn(bb, m1, t);       // fl(t - bb)
  const float2 d1 = __ffma2_rn(tb, m1, sh);      // fl(sh - (t - bb))
  const float2 s = __fadd2_rn(np, bb);           // -fl(p - bb)
  const float2 te = __ffma2_rn(s, m1, d1);       // the two-sum error fl(d1 + (p - bb))
  sl = __fadd2_rn(sl, __fadd2_rn(te, e));
  sh = t;
}

// FP32 -> FP64 from the bits (integer operations; GB300's FP64 pipe is ~1/64 of the FP32 rate):
// exact for normal floats, FP32 subnormals become 0.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xFFu;
  if (e == 0u) return 0.0;
  unsigned long long d = ((unsigned long long)(b & 0x80000000u) << 32) |
                         ((unsigned long long)(e == 255u ? 2047u : e + 896u) << 52) |
                         ((unsigned long long)(b & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}

}  // namespace fem
