// Double-float arithmetic for the complex128 passes.
//
// GB300 executes FP64 at about 2 lane-operations per clock per SM, 64 times
// below its FP32 rate, so a complex128 FFT in native FP64 is bound by the FP64
// pipe.  The passes of the default complex128 form keep the state in HBM as
// complex128 but do their arithmetic on unevaluated sums of two FP32 numbers
// (hi + lo, |lo| <= ulp(hi)/2), using the error-free transformations
//   TwoSum (Knuth, TAOCP vol. 2, 4.2.2)        a + b = s + e exactly
//   FastTwoSum (Dekker 1971), |a| >= |b|       a + b = s + e exactly
//   TwoProd with a fused multiply-add          a * b = p + e exactly
// on the FP32 pipes.  Products that feed an error-free transformation are
// written with __fmul_rn so that the compiler cannot contract them into a
// fused multiply-add.  Each operation carries about 2^-48 relative error (48
// significant bits against FP64's 53), which keeps an FFT of 8192 points
// within a few 1e-14 of the exact transform.  The exponent range is FP32's;
// values below about 1e-30 lose low-order bits, far below the tolerance of
// any quantity the propagators report.
#pragma once
#include <cuda_runtime.h>

struct __align__(8) dfr {
  float h, l;
};

// A complex number as two packed FP32 pairs, hi = (re hi, im hi) and lo = (re lo, im lo): sm_100 and
// later execute one FADD2 / FMUL2 / FFMA2 instruction on both lanes of a pair (each lane rounded
// exactly as the scalar instruction), so the real and imaginary parts of every double-float
// operation share their instructions.  In memory: (re hi, im hi, re lo, im lo), 16 bytes.
struct __align__(16) dfc {
  float2 h, l;
};

__device__ __forceinline__ dfr df_fast_two_sum(float a, float b) {
  const float s = a + b;
  return dfr{s, b - (s - a)};
}

__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ dfr df_add(dfr a, dfr b) {
  float s, e;
  df_two_sum(a.h, b.h, s, e);
  e += a.l + b.l;
  return df_fast_two_sum(s, e);
}

__device__ __forceinline__ dfr df_neg(dfr a) { return dfr{-a.h, -a.l}; }

// Sum without the final renormalisation (8 instead of 11 instructions): the pair (s, e + a.l + b.l)
// represents a + b to the same accuracy but its low part may exceed ulp(s) / 2.  A chain of such sums
// inside one butterfly is renormalised once at its end (df_renorm).
__device__ __forceinline__ dfr df_add_lazy(dfr a, dfr b) {
  float s, e;
  df_two_sum(a.h, b.h, s, e);
  return dfr{s, e + (a.l + b.l)};
}
__device__ __forceinline__ dfr df_sub_lazy(dfr a, dfr b) { return df_add_lazy(a, df_neg(b)); }
__device__ __forceinline__ dfr df_renorm(dfr a) { return df_fast_two_sum(a.h, a.l); }
__device__ __forceinline__ dfr df_sub(dfr a, dfr b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ dfr df_mul(dfr a, dfr b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_fast_two_sum(p, e);
}

// a*b - c*d without the final renormalisation (the real part of a complex product): the pair
// (s, e) represents the result as accurately as its renormalised form, with |e| up to a few ulp(s)
__device__ __forceinline__ dfr df_mul_sub_lazy(dfr a, dfr b, dfr c, dfr d) {
  const float p1 = __fmul_rn(a.h, b.h);
  const float e1 = __fmaf_rn(a.h, b.h, -p1);
  const float p2 = __fmul_rn(c.h, d.h);
  const float e2 = __fmaf_rn(c.h, d.h, -p2);
  float s, e;
  df_two_sum(p1, -p2, s, e);
  e += e1 - e2;
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  e = __fmaf_rn(-c.h, d.l, e);
  e = __fmaf_rn(-c.l, d.h, e);
  return dfr{s, e};
}
// a*b - c*d with one renormalisation
__device__ __forceinline__ dfr df_mul_sub(dfr a, dfr b, dfr c, dfr d) {
  const dfr r = df_mul_sub_lazy(a, b, c, d);
  return df_fast_two_sum(r.h, r.l);
}

// a*b + c*d
__device__ __forceinline__ dfr df_mul_add(dfr a, dfr b, dfr c, dfr d) {
  return df_mul_sub(a, b, df_neg(c), d);
}

__device__ __forceinline__ dfr df_from_double(double v) {
  const float h = __double2float_rn(v);
  return dfr{h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double df_to_double(dfr a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ dfr df_from_float(float v) { return dfr{v, 0.f}; }

// ---------------------------------------------------------------- packed pairs
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __fadd2_rn(a, p_neg(b)); }
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 p_bcast(float a) { return make_float2(a, a); }
// (-y, x): multiplication of (x, y) by +i
__device__ __forceinline__ float2 p_rot(float2 a) { return make_float2(-a.y, a.x); }
// (y, x)
__device__ __forceinline__ float2 p_swap(float2 a) { return make_float2(a.y, a.x); }
// (x, -y)
__device__ __forceinline__ float2 p_conj(float2 a) { return make_float2(a.x, -a.y); }

// TwoSum on both lanes: a + b = s + e exactly
__device__ __forceinline__ void p_two_sum(float2 a, float2 b, float2& s, float2& e) {
  s = p_add(a, b);
  const float2 bb = p_sub(s, a);
  e = p_add(p_sub(a, p_sub(s, bb)), p_sub(b, bb));
}
// a - b = s + e exactly
__device__ __forceinline__ void p_two_diff(float2 a, float2 b, float2& s, float2& e) {
  s = p_sub(a, b);
  const float2 bb = p_sub(s, a);  // -b, rounded
  e = p_sub(p_sub(a, p_sub(s, bb)), p_add(b, bb));
}

// ---------------------------------------------------------------- complex double-float
__device__ __forceinline__ dfr dfc_re(dfc a) { return dfr{a.h.x, a.l.x}; }
__device__ __forceinline__ dfr dfc_im(dfc a) { return dfr{a.h.y, a.l.y}; }
__device__ __forceinline__ dfc dfc_make(dfr re, dfr im) {
  return dfc{make_float2(re.h, im.h), make_float2(re.l, im.l)};
}
__device__ __forceinline__ dfc dfc_from_double2(double2 v) { return dfc_make(df_from_double(v.x), df_from_double(v.y)); }
__device__ __forceinline__ double2 dfc_to_double2(dfc v) {
  return make_double2((double)v.h.x + (double)v.l.x, (double)v.h.y + (double)v.l.y);
}

// sums without the final renormalisation (the pair's low part may exceed ulp(hi) / 2); a chain of
// them inside one butterfly is renormalised once at its end (dfc_renorm)
__device__ __forceinline__ dfc dfc_add_lazy(dfc a, dfc b) {
  float2 s, e;
  p_two_sum(a.h, b.h, s, e);
  return dfc{s, p_add(e, p_add(a.l, b.l))};
}
__device__ __forceinline__ dfc dfc_sub_lazy(dfc a, dfc b) {
  float2 s, e;
  p_two_diff(a.h, b.h, s, e);
  return dfc{s, p_add(e, p_sub(a.l, b.l))};
}
// FastTwoSum of (hi, lo) on both lanes
__device__ __forceinline__ dfc dfc_renorm(dfc a) {
  const float2 s = p_add(a.h, a.l);
  return dfc{s, p_sub(a.l, p_sub(s, a.h))};
}
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return dfc_renorm(dfc_add_lazy(a, b)); }
__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) { return dfc_renorm(dfc_sub_lazy(a, b)); }

// x * u + y * v on both lanes for x, y given as scalars (broadcast) and u, v as pairs, without the
// final renormalisation: TwoProd of the high parts, TwoSum of the two products, and the cross terms
// of the low parts (the lo * lo terms are below the working precision)
__device__ __forceinline__ dfc p_dot2_lazy(dfr x, float2 uh, float2 ul, dfr y, float2 vh, float2 vl) {
  const float2 xh = p_bcast(x.h), yh = p_bcast(y.h);
  const float2 p = p_mul(xh, uh);
  const float2 ep = p_fma(xh, uh, p_neg(p));
  const float2 q = p_mul(yh, vh);
  const float2 eq = p_fma(yh, vh, p_neg(q));
  float2 s, e;
  p_two_sum(p, q, s, e);
  e = p_add(e, p_add(ep, eq));
  e = p_fma(xh, ul, e);
  e = p_fma(p_bcast(x.l), uh, e);
  e = p_fma(yh, vl, e);
  e = p_fma(p_bcast(y.l), vh, e);
  return dfc{s, e};
}
// a * b = re(a) (b.re, b.im) + im(a) (-b.im, b.re)
__device__ __forceinline__ dfc dfc_mul_lazy(dfc a, dfc b) {
  return p_dot2_lazy(dfc_re(a), b.h, b.l, dfc_im(a), p_rot(b.h), p_rot(b.l));
}
// a * conj(b) = re(a) (b.re, -b.im) + im(a) (b.im, b.re)
__device__ __forceinline__ dfc dfc_mulc_lazy(dfc a, dfc b) {
  return p_dot2_lazy(dfc_re(a), p_conj(b.h), p_conj(b.l), dfc_im(a), p_swap(b.h), p_swap(b.l));
}
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) { return dfc_renorm(dfc_mul_lazy(a, b)); }
__device__ __forceinline__ dfc dfc_mulc(dfc a, dfc b) { return dfc_renorm(dfc_mulc_lazy(a, b)); }
// a * s for a double-float real s
__device__ __forceinline__ dfc dfc_scale_lazy(dfc a, dfr s) {
  const float2 sh = p_bcast(s.h);
  const float2 p = p_mul(a.h, sh);
  float2 e = p_fma(a.h, sh, p_neg(p));
  e = p_fma(a.h, p_bcast(s.l), e);
  e = p_fma(a.l, sh, e);
  return dfc{p, e};
}
__device__ __forceinline__ dfc dfc_scale(dfc a, dfr s) { return dfc_renorm(dfc_scale_lazy(a, s)); }
// |a|^2 as a double-float real
__device__ __forceinline__ dfr dfc_abs2(dfc a) {
  const float2 p = p_mul(a.h, a.h);
  float2 e = p_fma(a.h, a.h, p_neg(p));
  e = p_fma(p_add(a.h, a.h), a.l, e);
  return df_add(dfr{p.x, e.x}, dfr{p.y, e.y});
}
