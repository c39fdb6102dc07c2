// aw_reduce_noalloc: the deterministic buffer reduction of aw_sum / aw_purity /
// aw_trace, for callers that must not allocate device memory.
//
// Who cannot allocate: a host application that owns the whole device memory
// budget (a serving process that reserves HBM up front and hands this library
// only pointers into its own pool), and latency-critical loops in which a
// cudaMalloc / cudaFree would synchronise the device and stall work queued on
// other streams.  Such callers pass their own input and output pointers; the
// only scratch this entry point touches is the fixed array below.
//
// Scratch: one double2 partial sum per chunk of AW_NOALLOC_CHUNK elements, in a
// file-scope __device__ array of AW_NOALLOC_MAX_CHUNKS entries (16 KiB).  Every
// GPU that loads this library holds it until the process exits.  All calls on a
// device share it and it keeps the last call's partials; each call writes every
// partial it later reads, so nothing has to start at zero.  Calls whose kernels
// overlap on the GPU (different streams without ordering) race on the array.
//
// The first call made on a device does the set-up: with that device current it
// looks up the array's device address (cudaGetSymbolAddress) and keeps it for
// later calls.  Make that first call on each device before any stream capture.
// Later calls made outside stream capture look the address up again (cheap once
// the module is loaded), so a cudaDeviceReset, after which the array lives at a
// new address, is followed; a call made while its stream is being captured uses
// the address kept by the last call outside capture.
#include <cuda_runtime.h>

#include <stdint.h>

#include <mutex>
#include <string>

#include "awigner.h"

// records the message aw_last_error() returns (aw_api.cu)
void aw_internal_set_error(const char* msg);

#define AW_NOALLOC_CHUNK 65536LL
#define AW_NOALLOC_MAX_CHUNKS 1024
#define AW_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double2 aw_noalloc_partials[AW_NOALLOC_MAX_CHUNKS];

namespace {

std::mutex g_setup_mu;
double2* g_partials[AW_NOALLOC_MAX_DEVICES] = {nullptr};

int nofail(int code, const std::string& msg) {
  aw_internal_set_error(msg.c_str());
  return code;
}

__device__ __forceinline__ double2 ldv(const void* p, long long k, int f32) {
  if (f32) {
    const float2 v = ((const float2*)p)[k];
    return make_double2(v.x, v.y);
  }
  return ((const double2*)p)[k];
}

// block b reduces elements [b * CHUNK, min(n, (b + 1) * CHUNK)) in a fixed order
__global__ void k_chunk_partial(const void* a, int f32, long long n, int mode, long long stride, double2* part) {
  __shared__ double rr[256], ri[256];
  const long long lo = (long long)blockIdx.x * AW_NOALLOC_CHUNK;
  const long long hi = lo + AW_NOALLOC_CHUNK < n ? lo + AW_NOALLOC_CHUNK : n;
  double sr = 0.0, si = 0.0;
  for (long long k = lo + threadIdx.x; k < hi; k += blockDim.x) {
    const double2 v = ldv(a, mode == 3 ? k * stride : k, f32);
    if (mode == 0 || mode == 3) {
      sr += v.x;
      si += v.y;
    } else if (mode == 1) {
      sr += v.x * v.x - v.y * v.y;
    } else {
      sr += v.x * v.x + v.y * v.y;
    }
  }
  const int t = threadIdx.x;
  rr[t] = sr;
  ri[t] = si;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      rr[t] += rr[t + w];
      ri[t] += ri[t + w];
    }
    __syncthreads();
  }
  if (t == 0) part[blockIdx.x] = make_double2(rr[0], ri[0]);
}

// one block sums the partials in index order into the caller's output
__global__ void k_chunk_final(const double2* part, int nchunks, double* out) {
  __shared__ double rr[256], ri[256];
  double sr = 0.0, si = 0.0;
  for (int k = threadIdx.x; k < nchunks; k += blockDim.x) {
    sr += part[k].x;
    si += part[k].y;
  }
  const int t = threadIdx.x;
  rr[t] = sr;
  ri[t] = si;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      rr[t] += rr[t + w];
      ri[t] += ri[t + w];
    }
    __syncthreads();
  }
  if (t == 0) {
    out[0] = rr[0];
    out[1] = ri[0];
  }
}

}  // namespace

extern "C" int aw_reduce_noalloc(const void* data, int32_t elem_bytes, int64_t n, int64_t stride, int32_t mode,
                                 double* out_device, void* stream) {
  if (!out_device || (n > 0 && !data)) return nofail(AW_E_ARG, "aw_reduce_noalloc: null pointer");
  if (elem_bytes != 16 && elem_bytes != 8)
    return nofail(AW_E_ARG, "aw_reduce_noalloc: elem_bytes must be 16 (complex128) or 8 (complex64)");
  if (mode < 0 || mode > 3) return nofail(AW_E_ARG, "aw_reduce_noalloc: mode must be 0, 1, 2 or 3");
  if (n < 0) return nofail(AW_E_ARG, "aw_reduce_noalloc: negative element count");
  if (n > AW_NOALLOC_CHUNK * AW_NOALLOC_MAX_CHUNKS)
    return nofail(AW_E_ARG, "aw_reduce_noalloc: at most 67108864 elements (1024 chunks of 65536, the size of its "
                            "static scratch); got " + std::to_string((long long)n));
  if (mode == 3 && stride <= 0) return nofail(AW_E_ARG, "aw_reduce_noalloc: the trace needs a positive stride");
  // the trace reads element (n - 1) * stride: that index must exist as a 64-bit integer
  if (mode == 3 && n > 1 && stride > (INT64_MAX / (n - 1)))
    return nofail(AW_E_ARG, "aw_reduce_noalloc: (n - 1) * stride overflows a 64-bit index");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nofail(AW_E_CUDA, std::string("aw_reduce_noalloc: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= AW_NOALLOC_MAX_DEVICES) return nofail(AW_E_ARG, "aw_reduce_noalloc: device index too large");
  cudaStream_t st = (cudaStream_t)stream;
  // outside capture the address is looked up (again); inside, the kept one is used
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  const cudaError_t qe = cudaStreamIsCapturing(st, &cap);
  if (qe != cudaSuccess) cudaGetLastError();  // a refused query (capture elsewhere) leaves no error behind
  const bool capturing = qe != cudaSuccess || cap != cudaStreamCaptureStatusNone;
  double2* part;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_partials[dev] || !capturing) {
      if (capturing)
        return nofail(AW_E_ARG, "aw_reduce_noalloc: the first call on a device must come before stream capture");
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, aw_noalloc_partials);
      if (e != cudaSuccess)
        return nofail(AW_E_CUDA, std::string("aw_reduce_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_partials[dev] = (double2*)p;
    }
    part = g_partials[dev];
  }
  const int nchunks = (int)((n + AW_NOALLOC_CHUNK - 1) / AW_NOALLOC_CHUNK);
  if (nchunks > 0) k_chunk_partial<<<nchunks, 256, 0, st>>>(data, elem_bytes == 8, n, mode, stride, part);
  k_chunk_final<<<1, 256, 0, st>>>(part, nchunks, out_device);
  e = cudaGetLastError();
  if (e != cudaSuccess) return nofail(AW_E_CUDA, std::string("aw_reduce_noalloc: launch: ") + cudaGetErrorString(e));
  return AW_OK;
}
