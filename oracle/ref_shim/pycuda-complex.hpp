// CPU stand-in for the two CUDA facilities the reference's kernel templates use.
// TEST INFRASTRUCTURE ONLY (oracle/ref_build.py): pycuda::complex<double> becomes
// std::complex<double>, and the CUDA built-in thread indices become globals that a
// generated launcher loops over.
#pragma once
#include <cmath>
#include <complex>
#include <cstddef>

namespace pycuda {
template <class T>
using complex = std::complex<T>;
}
using std::abs;
using std::conj;
using std::exp;
using std::pow;
using std::sqrt;
using std::log;
using std::sin;
using std::cos;

struct aw_ref_dim3 {
  size_t x, y, z;
};
extern aw_ref_dim3 blockIdx, threadIdx, blockDim;

#define __global__
#define __device__ static inline
