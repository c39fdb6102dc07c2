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

struct __align__(16) dfc {
  dfr x, y;  // real and imaginary parts
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

__device__ __forceinline__ dfc dfc_from_double2(double2 v) { return dfc{df_from_double(v.x), df_from_double(v.y)}; }
__device__ __forceinline__ double2 dfc_to_double2(dfc v) { return make_double2(df_to_double(v.x), df_to_double(v.y)); }

// complex operations used by the FFT and the factors
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return dfc{df_add(a.x, b.x), df_add(a.y, b.y)}; }
__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) { return dfc{df_sub(a.x, b.x), df_sub(a.y, b.y)}; }
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
  return dfc{df_mul_sub(a.x, b.x, a.y, b.y), df_mul_add(a.x, b.y, a.y, b.x)};
}
// a * conj(b)
__device__ __forceinline__ dfc dfc_mulc(dfc a, dfc b) {
  return dfc{df_mul_add(a.x, b.x, a.y, b.y), df_mul_sub(a.y, b.x, a.x, b.y)};
}
__device__ __forceinline__ dfc dfc_scale(dfc a, dfr s) { return dfc{df_mul(a.x, s), df_mul(a.y, s)}; }
// complex products without the final renormalisation, for chains that end in one (df_renorm)
__device__ __forceinline__ dfc dfc_mul_lazy(dfc a, dfc b) {
  return dfc{df_mul_sub_lazy(a.x, b.x, a.y, b.y), df_mul_sub_lazy(a.x, b.y, df_neg(a.y), b.x)};
}
__device__ __forceinline__ dfc dfc_mulc_lazy(dfc a, dfc b) {
  return dfc{df_mul_sub_lazy(a.x, b.x, df_neg(a.y), b.y), df_mul_sub_lazy(a.y, b.x, a.x, b.y)};
}
__device__ __forceinline__ dfc dfc_add_lazy(dfc a, dfc b) { return dfc{df_add_lazy(a.x, b.x), df_add_lazy(a.y, b.y)}; }
__device__ __forceinline__ dfc dfc_sub_lazy(dfc a, dfc b) { return dfc{df_sub_lazy(a.x, b.x), df_sub_lazy(a.y, b.y)}; }
__device__ __forceinline__ dfc dfc_renorm(dfc a) { return dfc{df_renorm(a.x), df_renorm(a.y)}; }
