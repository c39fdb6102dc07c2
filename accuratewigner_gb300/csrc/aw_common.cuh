// Complex helpers shared by the sm_103a pass kernels.
//
// The reference keeps every state in pycuda::complex<double>
// (wigner_moyal_cuda_1d.py:629); here a state element is a CUDA vector type:
// double2 for the native complex128 form, float2 for the complex64 form and
// dfc (a double-float complex of two packed FP32 pairs, also 16 bytes) for the
// complex128 form computed on the FP32 pipes.  Element-wise code reads the
// parts through cre / cim and builds elements with cmake.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "aw_df.cuh"

// devices one process can drive (per-device records of the launchers)
#define AW_MAX_DEVICES 64

// Number of SMs of the current device, looked up once per device; grids are sized in multiples of
// it (152 on GB300).
inline int aw_sm_count() {
  static std::atomic<int> cache[AW_MAX_DEVICES];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= AW_MAX_DEVICES) return 1;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return 1;
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

template <typename T> struct cvec;
template <> struct cvec<double> { typedef double2 type; };
template <> struct cvec<float> { typedef float2 type; };

template <typename V> struct scalar_of;
template <> struct scalar_of<double2> { typedef double type; };
template <> struct scalar_of<float2> { typedef float type; };
template <> struct scalar_of<dfc> { typedef dfr type; };

// double-float scalar operators, so that the element-wise code is written once
__device__ __forceinline__ dfr operator+(dfr a, dfr b) { return df_add(a, b); }
__device__ __forceinline__ dfr operator-(dfr a, dfr b) { return df_sub(a, b); }
__device__ __forceinline__ dfr operator-(dfr a) { return df_neg(a); }
__device__ __forceinline__ dfr operator*(dfr a, dfr b) { return df_mul(a, b); }
__device__ __forceinline__ dfr& operator*=(dfr& a, dfr b) { return a = df_mul(a, b); }
__device__ __forceinline__ dfr& operator+=(dfr& a, dfr b) { return a = df_add(a, b); }
__device__ __forceinline__ dfr& operator-=(dfr& a, dfr b) { return a = df_sub(a, b); }
__device__ __forceinline__ bool operator==(dfr a, dfr b) { return a.h == b.h && a.l == b.l; }

// scalar conversions
template <typename T> __device__ __forceinline__ T from_double(double v) { return (T)v; }
template <> __device__ __forceinline__ dfr from_double<dfr>(double v) { return df_from_double(v); }
__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(float v) { return (double)v; }
__device__ __forceinline__ double to_d(dfr v) { return df_to_double(v); }

// lanes of a warp that exist in a block of NT threads
template <int NT> __device__ __forceinline__ unsigned lane_mask() { return NT >= 32 ? 0xffffffffu : (1u << NT) - 1u; }

// warp shuffles of a scalar over the lanes in m
__device__ __forceinline__ double shfl_xor(unsigned m, double v, int o, int w) { return __shfl_xor_sync(m, v, o, w); }
__device__ __forceinline__ float shfl_xor(unsigned m, float v, int o, int w) { return __shfl_xor_sync(m, v, o, w); }
__device__ __forceinline__ dfr shfl_xor(unsigned m, dfr v, int o, int w) {
  return dfr{__shfl_xor_sync(m, v.h, o, w), __shfl_xor_sync(m, v.l, o, w)};
}

// accumulator of per-thread partial sums (at most 16 terms; FP64 across threads): FP64 for double2,
// double-float for dfc, FP32 for float2 -- an FP64 operation per element runs at GB300's FP64 rate
// (2 lanes a clock a SM) and made the complex64 4096^2 reduction pass FP64-bound (241 us)
template <typename V> struct acc_of { typedef double type; };
template <> struct acc_of<dfc> { typedef dfr type; };
template <> struct acc_of<float2> { typedef float type; };
template <typename A> __device__ __forceinline__ A to_acc(double v) { return from_double<A>(v); }
template <typename A> __device__ __forceinline__ A to_acc(float v) { return (A)(double)v; }
template <> __device__ __forceinline__ dfr to_acc<dfr>(float v) { return df_from_float(v); }
template <typename A> __device__ __forceinline__ A to_acc(dfr v);
template <> __device__ __forceinline__ dfr to_acc<dfr>(dfr v) { return v; }

// partial sums exchanged between the blocks of a cluster: FP64 for the native types, the working
// double-float form for dfc (converted to FP64 once, after the cluster sum)
template <typename V> struct cpart {
  typedef double2 type;
  __device__ static double2 make(typename scalar_of<V>::type x, typename scalar_of<V>::type y) {
    return make_double2(to_d(x), to_d(y));
  }
  __device__ static double2 zero() { return make_double2(0.0, 0.0); }
  __device__ static double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
  __device__ static double2 to_d2(double2 a) { return a; }
  __device__ static double2 shfl_xor(unsigned m, double2 a, int o, int w) {
    return make_double2(__shfl_xor_sync(m, a.x, o, w), __shfl_xor_sync(m, a.y, o, w));
  }
};
template <> struct cpart<dfc> {
  typedef dfc type;
  __device__ static dfc make(dfr x, dfr y) { return dfc_make(x, y); }
  __device__ static dfc zero() { return dfc{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
  __device__ static dfc add(dfc a, dfc b) { return dfc_add(a, b); }
  __device__ static double2 to_d2(dfc a) { return dfc_to_double2(a); }
  __device__ static dfc shfl_xor(unsigned m, dfc a, int o, int w) {
    return dfc{make_float2(__shfl_xor_sync(m, a.h.x, o, w), __shfl_xor_sync(m, a.h.y, o, w)),
               make_float2(__shfl_xor_sync(m, a.l.x, o, w), __shfl_xor_sync(m, a.l.y, o, w))};
  }
};

template <typename V>
__device__ __forceinline__ V cmake(typename scalar_of<V>::type x, typename scalar_of<V>::type y) {
  V r;
  r.x = x;
  r.y = y;
  return r;
}
template <> __device__ __forceinline__ dfc cmake<dfc>(dfr x, dfr y) { return dfc_make(x, y); }

// real and imaginary parts
template <typename V> __device__ __forceinline__ typename scalar_of<V>::type cre(V a) { return a.x; }
template <typename V> __device__ __forceinline__ typename scalar_of<V>::type cim(V a) { return a.y; }
template <> __device__ __forceinline__ dfr cre<dfc>(dfc a) { return dfc_re(a); }
template <> __device__ __forceinline__ dfr cim<dfc>(dfc a) { return dfc_im(a); }

// |a|^2 in the working precision
template <typename V> __device__ __forceinline__ typename scalar_of<V>::type cabs2(V a) {
  return a.x * a.x + a.y * a.y;
}
template <> __device__ __forceinline__ dfr cabs2<dfc>(dfc a) { return dfc_abs2(a); }

template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return cmake<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return cmake<V>(a.x - b.x, a.y - b.y); }

// a * b
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  return cmake<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// a * conj(b)
template <typename V> __device__ __forceinline__ V cmulc(V a, V b) {
  return cmake<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

template <typename V> __device__ __forceinline__ V cscale(V a, typename scalar_of<V>::type s) {
  return cmake<V>(a.x * s, a.y * s);
}

// complex64 on packed FP32 pairs: one FADD2 for a sum, FMUL2 + FFMA2 for a product
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) { return __fadd2_rn(a, b); }
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) { return __fadd2_rn(a, p_neg(b)); }
// a b = re(a) (b.x, b.y) + im(a) (-b.y, b.x)
template <> __device__ __forceinline__ float2 cmul<float2>(float2 a, float2 b) {
  return __ffma2_rn(p_bcast(a.x), b, __fmul2_rn(p_bcast(a.y), p_rot(b)));
}
// a conj(b) = re(a) (b.x, -b.y) + im(a) (b.y, b.x)
template <> __device__ __forceinline__ float2 cmulc<float2>(float2 a, float2 b) {
  return __ffma2_rn(p_bcast(a.x), p_conj(b), __fmul2_rn(p_bcast(a.y), p_swap(b)));
}
template <> __device__ __forceinline__ float2 cscale<float2>(float2 a, float s) { return __fmul2_rn(a, p_bcast(s)); }

template <> __device__ __forceinline__ dfc cadd<dfc>(dfc a, dfc b) { return dfc_add(a, b); }
template <> __device__ __forceinline__ dfc csub<dfc>(dfc a, dfc b) { return dfc_sub(a, b); }
template <> __device__ __forceinline__ dfc cmul<dfc>(dfc a, dfc b) { return dfc_mul(a, b); }
template <> __device__ __forceinline__ dfc cmulc<dfc>(dfc a, dfc b) { return dfc_mulc(a, b); }
template <> __device__ __forceinline__ dfc cscale<dfc>(dfc a, dfr s) { return dfc_scale(a, s); }

// sign flips by a mask of the sign bit (0 or 0x80000000), on the integer pipe
__device__ __forceinline__ float flip(float v, unsigned m) { return __int_as_float(__float_as_int(v) ^ (int)m); }
__device__ __forceinline__ double flip(double v, unsigned m) {
  return __longlong_as_double(__double_as_longlong(v) ^ (long long)((unsigned long long)m << 32));
}
__device__ __forceinline__ dfr flip(dfr v, unsigned m) { return dfr{flip(v.h, m), flip(v.l, m)}; }
__device__ __forceinline__ float2 flip(float2 v, unsigned mx, unsigned my) { return make_float2(flip(v.x, mx), flip(v.y, my)); }
template <typename V> __device__ __forceinline__ V cflip(V a, unsigned m) { return cmake<V>(flip(a.x, m), flip(a.y, m)); }
template <typename V> __device__ __forceinline__ V cconj_if(V a, unsigned m) { return cmake<V>(a.x, flip(a.y, m)); }
template <> __device__ __forceinline__ dfc cflip<dfc>(dfc a, unsigned m) { return dfc{flip(a.h, m, m), flip(a.l, m, m)}; }
template <> __device__ __forceinline__ dfc cconj_if<dfc>(dfc a, unsigned m) { return dfc{flip(a.h, 0u, m), flip(a.l, 0u, m)}; }

// butterfly sums: for dfc without renormalisation (cnorm renormalises once at a butterfly's end);
// the same as cadd / csub for the native types
template <typename V> __device__ __forceinline__ V cadd_l(V a, V b) { return cadd(a, b); }
template <typename V> __device__ __forceinline__ V csub_l(V a, V b) { return csub(a, b); }
template <typename V> __device__ __forceinline__ V cnorm(V a) { return a; }
template <> __device__ __forceinline__ dfc cadd_l<dfc>(dfc a, dfc b) { return dfc_add_lazy(a, b); }
template <> __device__ __forceinline__ dfc csub_l<dfc>(dfc a, dfc b) { return dfc_sub_lazy(a, b); }
template <> __device__ __forceinline__ dfc cnorm<dfc>(dfc a) { return dfc_renorm(a); }
// products likewise: for dfc without renormalisation
template <typename V> __device__ __forceinline__ V cmul_l(V a, V b) { return cmul(a, b); }
template <typename V> __device__ __forceinline__ V cmulc_l(V a, V b) { return cmulc(a, b); }
template <> __device__ __forceinline__ dfc cmul_l<dfc>(dfc a, dfc b) { return dfc_mul_lazy(a, b); }
template <> __device__ __forceinline__ dfc cmulc_l<dfc>(dfc a, dfc b) { return dfc_mulc_lazy(a, b); }

// Transform direction of the FFT helpers: inv = 0 for the forward transform (exp(-i ...)),
// 0x80000000 for the inverse; the direction is a run-time value so that one copy of the code
// serves both.
// a * (-i) forward, a * (+i) inverse
template <typename V> __device__ __forceinline__ V cmul_mi_dir(V a, unsigned inv) {
  return cmake<V>(flip(a.y, inv), flip(a.x, inv ^ 0x80000000u));
}
template <> __device__ __forceinline__ dfc cmul_mi_dir<dfc>(dfc a, unsigned inv) {
  const unsigned m = inv ^ 0x80000000u;
  return dfc{flip(p_swap(a.h), inv, m), flip(p_swap(a.l), inv, m)};
}

// 1/sqrt(2) in the working type (double-float: the FP32 pair nearest to it)
template <typename T> __device__ __forceinline__ T rsqrt2() { return T(0.70710678118654752440); }
template <> __device__ __forceinline__ dfr rsqrt2<dfr>() { return dfr{0.70710677f, 1.21016175e-08f}; }

// a * exp(-+ i pi/4):  forward (x + y, y - x)/sqrt2, inverse (x - y, y + x)/sqrt2
template <typename V> __device__ __forceinline__ V cmul_w8_1_dir(V a, unsigned inv) {
  typedef typename scalar_of<V>::type T;
  const T h = rsqrt2<T>();
  return cmake<V>((a.x + flip(a.y, inv)) * h, (a.y - flip(a.x, inv)) * h);
}
// double-float: a + (y, -x) forward, a + (-y, x) inverse on both lanes, then the scale; the lazy
// sum feeds the product directly (its low part enters through the cross term) and one
// renormalisation ends it
template <> __device__ __forceinline__ dfc cmul_w8_1_dir<dfc>(dfc a, unsigned inv) {
  const unsigned m = inv ^ 0x80000000u;
  const dfc t = dfc{flip(p_swap(a.h), inv, m), flip(p_swap(a.l), inv, m)};  // a * (-+ i)
  return dfc_renorm(dfc_scale_lazy(dfc_add_lazy(a, t), rsqrt2<dfr>()));
}
// a * exp(-+ 3 i pi/4) = (a * exp(-+ i pi/4)) * (-+ i)
template <typename V> __device__ __forceinline__ V cmul_w8_3_dir(V a, unsigned inv) {
  return cmul_mi_dir(cmul_w8_1_dir(a, inv), inv);
}
