// Complex helpers shared by the sm_103a pass kernels.
//
// The reference keeps every state in pycuda::complex<double>
// (wigner_moyal_cuda_1d.py:629); here a state element is a CUDA vector type:
// double2 for the plain complex128 form and float2 for the complex64 form.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

template <typename T> struct cvec;
template <> struct cvec<double> { typedef double2 type; };
template <> struct cvec<float> { typedef float2 type; };

template <typename V> struct scalar_of;
template <> struct scalar_of<double2> { typedef double type; };
template <> struct scalar_of<float2> { typedef float type; };

template <typename V>
__device__ __forceinline__ V cmake(typename scalar_of<V>::type x, typename scalar_of<V>::type y) {
  V r;
  r.x = x;
  r.y = y;
  return r;
}

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

// a * (-i) and a * (+i)
template <typename V> __device__ __forceinline__ V cmul_mi(V a) { return cmake<V>(a.y, -a.x); }
template <typename V> __device__ __forceinline__ V cmul_pi(V a) { return cmake<V>(-a.y, a.x); }

// multiply by exp(-i*pi/4 * s) for the radix-8 inner twiddles:  (1 -+ i)/sqrt(2)
template <typename V, bool FWD> __device__ __forceinline__ V cmul_w8_1(V a) {
  typedef typename scalar_of<V>::type T;
  const T h = T(0.70710678118654752440);
  // FWD: a * (1 - i)/sqrt2 ; INV: a * (1 + i)/sqrt2
  return FWD ? cmake<V>((a.x + a.y) * h, (a.y - a.x) * h) : cmake<V>((a.x - a.y) * h, (a.y + a.x) * h);
}
template <typename V, bool FWD> __device__ __forceinline__ V cmul_w8_3(V a) {
  typedef typename scalar_of<V>::type T;
  const T h = T(0.70710678118654752440);
  // FWD: a * (-1 - i)/sqrt2 ; INV: a * (-1 + i)/sqrt2
  return FWD ? cmake<V>((a.y - a.x) * h, -(a.x + a.y) * h) : cmake<V>(-(a.x + a.y) * h, (a.x - a.y) * h);
}
