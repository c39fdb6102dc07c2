// Element-wise and reduction kernels that need no user expression.
//
// Reductions are deterministic: a fixed grid of blocks writes one partial
// each and the partials are summed in index order, so repeated runs (and a
// propagation run alone or inside a batch) give bit-identical scalars.
#include <cuda_runtime.h>
#include <stdint.h>

#include "aw_common.cuh"
#include "aw_util.h"

namespace {

// element formats: 0 complex128, 1 complex64, 2 double-float complex (re hi, im hi, re lo, im lo)
__device__ __forceinline__ double2 ld(const void* p, long long k, int f32) {
  if (f32 == 1) {
    float2 v = ((const float2*)p)[k];
    return make_double2(v.x, v.y);
  }
  if (f32 == 2) {
    float4 v = ((const float4*)p)[k];
    return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
  }
  return ((const double2*)p)[k];
}
__device__ __forceinline__ float2 df_split(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}
__device__ __forceinline__ void st(void* p, long long k, int f32, double2 v) {
  if (f32 == 1) {
    ((float2*)p)[k] = make_float2((float)v.x, (float)v.y);
  } else if (f32 == 2) {
    const float2 a = df_split(v.x), b = df_split(v.y);
    ((float4*)p)[k] = make_float4(a.x, b.x, a.y, b.y);
  } else {
    ((double2*)p)[k] = v;
  }
}

// sum of one value per thread over a block of whole warps: a fixed shuffle tree in each warp, then
// the warp sums in index order; the same result in every thread
__device__ __forceinline__ double blk_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
  __syncthreads();
  return r;
}

// a *= (re + i im) * ptr[2 inst .. 2 inst + 1]; instance inst = blockIdx.y holds n elements
__global__ void k_scale(void* a, int f32, long long n, double re, double im, const double* ptr) {
  const long long inst = blockIdx.y;
  double sr = re, si = im;
  if (ptr) {
    const double pr = ptr[2 * inst], pi = ptr[2 * inst + 1];
    sr = re * pr - im * pi;
    si = re * pi + im * pr;
  }
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    double2 v = ld(a, inst * n + k, f32);
    st(a, inst * n + k, f32, make_double2(v.x * sr - v.y * si, v.x * si + v.y * sr));
  }
}

// tables t = 0 .. count-1 of n complex entries, `stride` entries apart: entry k *= s[k] (real)
__global__ void k_scale_lines(void* tab, int fmt, const double* sv, int n, long long stride) {
  const long long t = blockIdx.y;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double2 v = ld(tab, t * stride + k, fmt);
    const double f = sv[k];
    st(tab, t * stride + k, fmt, make_double2(v.x * f, v.y * f));
  }
}

__global__ void k_fill(void* a, int f32, long long n, double re, double im) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    st(a, k, f32, make_double2(re, im));
}

__global__ void k_convert(const void* src, int sf32, void* dst, int df32, long long n) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    st(dst, k, df32, ld(src, k, sf32));
}

// mode 0: sum of a; 1: sum of Re(a*a); 2: sum of |a|^2; 3: trace (n = N, stride N+1)
__global__ void k_partial(const void* a, int f32, long long n, int mode, long long stride, double2* part) {
  __shared__ double rr[256], ri[256];
  double sr = 0.0, si = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    double2 v = ld(a, mode == 3 ? k * stride : k, f32);
    if (mode == 0 || mode == 3) {
      sr += v.x;
      si += v.y;
    } else if (mode == 1) {
      sr += v.x * v.x - v.y * v.y;
    } else {
      sr += v.x * v.x + v.y * v.y;
    }
  }
  const double tr = blk_sum(sr, rr), ti = blk_sum(si, ri);
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(tr, ti);
}

__global__ void k_embed(const void* rho, int f32, int N, void* W, int M, int pad) {
  const long long n = (long long)M * M;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k / M), j = (int)(k - (long long)i * M);
    double2 v = make_double2(0.0, 0.0);
    if (i >= pad && i < pad + N && j >= pad && j < pad + N) v = ld(rho, (long long)(i - pad) * N + (j - pad), f32);
    st(W, k, f32, v);
  }
}

__global__ void k_psi2rho(const void* psi, int f32, int N, void* rho) {
  const long long n = (long long)N * N;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(k / N), j = (int)(k - (long long)i * N);
    const double2 a = ld(psi, j, f32), b = ld(psi, i, f32);
    // psi[j] * conj(psi[i])   (schrodinger_wigner_cuda_1d.py:680-687)
    st(rho, k, f32, make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y));
  }
}

// von Neumann / rho-Bloch per-step normalisation from the diagonal gathered by
// the row pass:  inv = 1 / (Re Tr rho * dX)  (rho_vneumann_cuda_1d.py:443) or
// 1 / (Tr rho * dX) with the complex trace (rho_bloch_cuda_1d.py:244).  The
// purity Sum |rho|^2 dX^2 (rho_vneumann_cuda_1d.py:565-579) of the normalised
// state follows from the row pass's |rho|^2 partials.
// blockIdx.x = instance: diag n apart, abs2part nparts apart, inv_out 2 apart, hist hstride apart
// trace (and purity) of one instance: 1 / trace into inv_out, the purity and trace into hist
__device__ __forceinline__ void trace_body(const double2* diag, int n, const double* abs2part, int nparts, double dX,
                                           int complex_trace, double* inv_out, double* hist, int* stop,
                                           int stop_on_purity) {
  __shared__ double rr[256], ri[256], ra[256];
  if (stop && *stop) return;
  const int t = threadIdx.x;
  double sr = 0.0, si = 0.0, sa = 0.0;
  for (int k = t; k < n; k += blockDim.x) {
    sr += diag[k].x;
    si += diag[k].y;
  }
  if (abs2part)
    for (int k = t; k < nparts; k += blockDim.x) sa += abs2part[k];
  sr = blk_sum(sr, rr);
  si = blk_sum(si, ri);
  sa = blk_sum(sa, ra);
  if (t == 0) {
    const double tr = sr * dX, ti = complex_trace ? si * dX : 0.0;
    const double d = tr * tr + ti * ti;
    const double ir = tr / d, ii = -ti / d;
    inv_out[0] = ir;
    inv_out[1] = ii;
    const double purity = sa * (ir * ir + ii * ii) * dX * dX;
    if (hist) {
      hist[0] = purity;
      hist[1] = tr;
      hist[2] = ti;
    }
    if (stop && stop_on_purity && !(purity < 1.0)) *stop = 1;
  }
}

__global__ void k_trace_finalize(const double2* diag, int n, const double* abs2part, int nparts, double dX,
                                 int complex_trace, double* inv_out, double* hist, long long hstride, int* stop,
                                 int stop_on_purity) {
  const long long in = blockIdx.x;
  trace_body(diag + in * n, n, abs2part ? abs2part + in * nparts : nullptr, nparts, dX, complex_trace,
             inv_out + 2 * in, hist ? hist + in * hstride : nullptr, stop ? stop + in : nullptr, stop_on_purity);
}

// the traces of the instances of several propagators: blockIdx.y member, blockIdx.x instance
__global__ void k_trace_finalize_group(const AwTraceGroup g) {
  const int m = blockIdx.y, in = blockIdx.x;
  if (in >= g.ninst[m]) return;
  const int n = g.n[m];
  trace_body(g.diag[m] + (long long)in * n, n, nullptr, 0, g.dX[m], g.complex_trace, g.inv[m] + 2 * in, nullptr,
             g.stop[m] ? g.stop[m] + in : nullptr, 0);
}

// 1 / sqrt(Sum parts * scale): renormalisation of a wave function
// (schrodinger_wigner_cuda_1d.py:388: psi /= norm(psi) * sqrt(dX))
__global__ void k_norm_finalize(const double* parts, int nparts, double scale, double* inv_out, double* hist) {
  __shared__ double r[256];
  const int t = threadIdx.x;
  double s = 0.0;
  for (int k = t; k < nparts; k += blockDim.x) s += parts[k];
  s = blk_sum(s, r);
  if (t == 0) {
    inv_out[0] = 1.0 / sqrt(s * scale);
    inv_out[1] = 0.0;
    if (hist) hist[0] = s;
  }
}

// |a|^2 as a real array
// |a_k|^2; with n1 > 0, a holds a spectrum in the four-step order (k = k1 + n1 k2 at k1 n2 + k2)
__global__ void k_abs2(const void* a, int f32, long long n, double* out, int n1) {
  const long long n2 = n1 > 0 ? n / n1 : 0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    double2 v = ld(a, n1 > 0 ? (k % n1) * n2 + k / n1 : k, f32);
    out[k] = v.x * v.x + v.y * v.y;
  }
}

// out[k] = a[(k % n1) n2 + k / n1]: a four-step spectrum into natural order
__global__ void k_unpermute(const void* a, void* out, int f32, long long n, int n1) {
  const long long n2 = n / n1;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    st(out, k, f32, ld(a, (k % n1) * n2 + k / n1, f32));
}

// partial sums of conj(a) * b (the reference's vdot ReductionKernel, sw:524-530)
__global__ void k_vdot(const void* a, const void* b, int f32, long long n, double2* part) {
  __shared__ double rr[256], ri[256];
  double sr = 0.0, si = 0.0;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const double2 x = ld(a, k, f32), y = ld(b, k, f32);
    sr += x.x * y.x + x.y * y.y;
    si += x.x * y.y - x.y * y.x;
  }
  const double tr = blk_sum(sr, rr), ti = blk_sum(si, ri);
  if (threadIdx.x == 0) part[blockIdx.x] = make_double2(tr, ti);
}

// y += (cr + i ci) x  (the reference's projectout ElementwiseKernel with C = -proj, sw:532-535)
__global__ void k_axpy(void* y, const void* x, int f32, long long n, double cr, double ci) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const double2 a = ld(x, k, f32);
    double2 b = ld(y, k, f32);
    b.x += cr * a.x - ci * a.y;
    b.y += cr * a.y + ci * a.x;
    st(y, k, f32, b);
  }
}

// out[k] = Sum_b part[b][k] in index order (partials of the column-pass cross reductions)
__global__ void k_sum_parts(const double2* part, int nparts, int n, double2* out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double sr = 0.0, si = 0.0;
  for (int b = 0; b < nparts; ++b) {
    const double2 v = part[(long long)b * n + k];
    sr += v.x;
    si += v.y;
  }
  out[k] = make_double2(sr, si);
}

// full[l][q] = hi[l][q / lo_n] * lo[l][q % lo_n] (complex128)
__global__ void k_shear_full(const double2* hi, const double2* lo, int lo_n, int lines, int npos, double2* full) {
  const long long n = (long long)lines * npos;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(k / npos), q = (int)(k % npos);
    const double2 a = hi[(long long)l * (npos / lo_n) + q / lo_n], b = lo[(long long)l * lo_n + q % lo_n];
    full[k] = make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
  }
}

// A separable factor as one table of conj(row[i]) * (scale * col[j]) (complex128), the product a tile
// otherwise forms from its line's constant and the table along the line: per column line j and
// position (row) i, full[j][i], for a column pass; per row line i and position j, full[i][j], for a
// row pass (row_lines)
__global__ void k_sep_full(const double2* col, const double2* row, double scale, int nr, int nc, int row_lines,
                           double2* full) {
  const long long n = (long long)nr * nc;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int j = row_lines ? (int)(k % nc) : (int)(k / nr), i = row_lines ? (int)(k / nc) : (int)(k % nr);
    const double2 c = make_double2(scale * col[j].x, scale * col[j].y), r = row[i];
    full[k] = make_double2(r.x * c.x + r.y * c.y, r.x * c.y - r.y * c.x);
  }
}

// The von Neumann momentum diagonal from the diagonal sums G of the branch point (aw_api.cu, vn_run):
// Re M_k = scale Re Sum_d G_d exp(-2 pi i k d / N), N = n1 n2, in two launches of direct FP64 DFTs
// (the four-step factorisation, d = d1 + n1 d2, k = k2 + n2 k1):
//   X[d1][k2] = exp(-2 pi i k2 d1 / N) Sum_d2 G[d1 + n1 d2] exp(-2 pi i k2 d2 / n2)     (block d1)
//   M[k2 + n2 k1] = scale Sum_d1 X[d1][k2] exp(-2 pi i k1 d1 / n1)                     (block k2)
// Twiddles from sincospi of exactly reduced integer ratios.  AW_DFT_PARTS threads share each output
// (interleaved terms, added in part order), so that the FP64 sums are short chains over more warps.
#define AW_DFT_PARTS 4
__global__ void k_diag_dft_a(const double2* g, int n1, int n2, double2* x) {
  extern __shared__ double2 aw_dsh[];
  double2* v = aw_dsh;
  double2* w = aw_dsh + n2;
  double2* part = aw_dsh + 2 * n2;  // [AW_DFT_PARTS][n2]
  const int d1 = blockIdx.x;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    v[t] = g[d1 + (long long)n1 * t];
    double sn, cs;
    sincospi(2.0 * t / n2, &sn, &cs);
    w[t] = make_double2(cs, -sn);
  }
  __syncthreads();
  for (int u = threadIdx.x; u < n2 * AW_DFT_PARTS; u += blockDim.x) {
    const int k2 = u % n2, q = u / n2;
    double re = 0.0, im = 0.0;
    for (int d2 = q; d2 < n2; d2 += AW_DFT_PARTS) {
      const double2 a = v[d2], b = w[(k2 * d2) & (n2 - 1)];
      re += a.x * b.x - a.y * b.y;
      im += a.x * b.y + a.y * b.x;
    }
    part[q * n2 + k2] = make_double2(re, im);
  }
  __syncthreads();
  const long long n = (long long)n1 * n2;
  for (int k2 = threadIdx.x; k2 < n2; k2 += blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int q = 0; q < AW_DFT_PARTS; ++q) {
      re += part[q * n2 + k2].x;
      im += part[q * n2 + k2].y;
    }
    double sn, cs;
    sincospi(2.0 * (double)(((long long)k2 * d1) % n) / (double)n, &sn, &cs);
    x[(long long)d1 * n2 + k2] = make_double2(re * cs + im * sn, im * cs - re * sn);
  }
}

__global__ void k_diag_dft_b(const double2* x, int n1, int n2, double scale, double* out_re) {
  extern __shared__ double2 aw_dsh[];
  double2* v = aw_dsh;
  double2* w = aw_dsh + n1;
  double* part = reinterpret_cast<double*>(aw_dsh + 2 * n1);  // [AW_DFT_PARTS][n1]
  const int k2 = blockIdx.x;
  for (int t = threadIdx.x; t < n1; t += blockDim.x) {
    v[t] = x[(long long)t * n2 + k2];
    double sn, cs;
    sincospi(2.0 * t / n1, &sn, &cs);
    w[t] = make_double2(cs, -sn);
  }
  __syncthreads();
  for (int u = threadIdx.x; u < n1 * AW_DFT_PARTS; u += blockDim.x) {
    const int k1 = u % n1, q = u / n1;
    double re = 0.0;
    for (int d1 = q; d1 < n1; d1 += AW_DFT_PARTS) {
      const double2 a = v[d1], b = w[(k1 * d1) & (n1 - 1)];
      re += a.x * b.x - a.y * b.y;
    }
    part[q * n1 + k1] = re;
  }
  __syncthreads();
  for (int k1 = threadIdx.x; k1 < n1; k1 += blockDim.x) {
    double re = 0.0;
    for (int q = 0; q < AW_DFT_PARTS; ++q) re += part[q * n1 + k1];
    out_re[k2 + (long long)n2 * k1] = scale * re;
  }
}

__global__ void k_set2(double* p, double a, double b) {
  p[0] = a;
  p[1] = b;
}

// grid-stride launches: at most 32 blocks of 256 threads per SM of the current device
inline int grid_for(long long n) {
  long long g = (n + 255) / 256;
  const long long cap = 32LL * aw_sm_count();
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

inline int ok() { return cudaGetLastError() == cudaSuccess ? 0 : -1; }

}  // namespace

extern "C" {

int aw_k_shear_full(const void* hi, const void* lo, int lo_n, int lines, int npos, void* full, void* s) {
  k_shear_full<<<grid_for((long long)lines * npos), 256, 0, (cudaStream_t)s>>>(
      (const double2*)hi, (const double2*)lo, lo_n, lines, npos, (double2*)full);
  return ok();
}

int aw_k_sep_full(const void* col, const void* row, double scale, int nr, int nc, int row_lines, void* full, void* s) {
  k_sep_full<<<grid_for((long long)nr * nc), 256, 0, (cudaStream_t)s>>>((const double2*)col, (const double2*)row, scale,
                                                                          nr, nc, row_lines, (double2*)full);
  return ok();
}

int aw_k_scale(void* a, int f32, long long n, double re, double im, const double* ptr, void* s) {
  return aw_k_scale_n(a, f32, n, 1, re, im, ptr, s);
}
int aw_k_scale_n(void* a, int f32, long long n, int ninst, double re, double im, const double* ptr, void* s) {
  const int gx = (grid_for(n) + ninst - 1) / ninst;
  k_scale<<<dim3(gx, ninst), 256, 0, (cudaStream_t)s>>>(a, f32, n, re, im, ptr);
  return ok();
}
int aw_k_scale_lines(void* tab, int fmt, const double* sv, int n, int count, long long stride, void* s) {
  k_scale_lines<<<dim3((n + 255) / 256, count), 256, 0, (cudaStream_t)s>>>(tab, fmt, sv, n, stride);
  return ok();
}
int aw_k_fill(void* a, int f32, long long n, double re, double im, void* s) {
  k_fill<<<grid_for(n), 256, 0, (cudaStream_t)s>>>(a, f32, n, re, im);
  return ok();
}
int aw_k_convert(const void* src, int sf32, void* dst, int df32, long long n, void* s) {
  k_convert<<<grid_for(n), 256, 0, (cudaStream_t)s>>>(src, sf32, dst, df32, n);
  return ok();
}
int aw_k_partial(const void* a, int f32, long long n, int mode, long long stride, double2* part, int nblocks, void* s) {
  k_partial<<<nblocks, 256, 0, (cudaStream_t)s>>>(a, f32, n, mode, stride, part);
  return ok();
}
int aw_k_embed(const void* rho, int f32, int N, void* W, int M, int pad, void* s) {
  k_embed<<<grid_for((long long)M * M), 256, 0, (cudaStream_t)s>>>(rho, f32, N, W, M, pad);
  return ok();
}
int aw_k_psi2rho(const void* psi, int f32, int N, void* rho, void* s) {
  k_psi2rho<<<grid_for((long long)N * N), 256, 0, (cudaStream_t)s>>>(psi, f32, N, rho);
  return ok();
}
int aw_k_trace_finalize(const double2* diag, int n, const double* abs2part, int nparts, double dX, int complex_trace,
                        double* inv_out, double* hist, int* stop, int stop_on_purity, void* s) {
  return aw_k_trace_finalize_n(diag, n, abs2part, nparts, dX, complex_trace, inv_out, hist, 0, stop, stop_on_purity, 1,
                               s);
}
int aw_k_trace_finalize_n(const double2* diag, int n, const double* abs2part, int nparts, double dX, int complex_trace,
                          double* inv_out, double* hist, long long hstride, int* stop, int stop_on_purity, int ninst,
                          void* s) {
  k_trace_finalize<<<ninst, 256, 0, (cudaStream_t)s>>>(diag, n, abs2part, nparts, dX, complex_trace, inv_out, hist,
                                                       hstride, stop, stop_on_purity);
  return ok();
}
int aw_k_diag_dft(const double2* g, int n, double2* scratch, double* out_re, double scale, void* s) {
  int l = 0;
  while ((1 << l) < n) ++l;
  if (n < 1 || (1 << l) != n) return -1;
  const int n1 = 1 << (l / 2), n2 = n / n1;
  const int ta = n2 * AW_DFT_PARTS < 256 ? n2 * AW_DFT_PARTS : 256;
  const int tb = n1 * AW_DFT_PARTS < 256 ? n1 * AW_DFT_PARTS : 256;
  k_diag_dft_a<<<n1, ta, (2 + AW_DFT_PARTS) * n2 * sizeof(double2), (cudaStream_t)s>>>(g, n1, n2, scratch);
  k_diag_dft_b<<<n2, tb, 2 * n1 * sizeof(double2) + AW_DFT_PARTS * n1 * sizeof(double), (cudaStream_t)s>>>(
      scratch, n1, n2, scale, out_re);
  return ok();
}
int aw_k_trace_finalize_group(const AwTraceGroup* g, void* s) {
  int most = 1;
  for (int m = 0; m < g->count; ++m) most = g->ninst[m] > most ? g->ninst[m] : most;
  k_trace_finalize_group<<<dim3(most, g->count), 256, 0, (cudaStream_t)s>>>(*g);
  return ok();
}
int aw_k_norm_finalize(const double* parts, int nparts, double scale, double* inv_out, double* hist, void* s) {
  k_norm_finalize<<<1, 256, 0, (cudaStream_t)s>>>(parts, nparts, scale, inv_out, hist);
  return ok();
}
int aw_k_abs2(const void* a, int f32, long long n, double* out, void* s) {
  k_abs2<<<grid_for(n), 256, 0, (cudaStream_t)s>>>(a, f32, n, out, 0);
  return ok();
}
int aw_k_abs2_perm(const void* a, int f32, long long n, int n1, double* out, void* s) {
  k_abs2<<<grid_for(n), 256, 0, (cudaStream_t)s>>>(a, f32, n, out, n1);
  return ok();
}
int aw_k_unpermute(const void* a, void* out, int f32, long long n, int n1, void* s) {
  k_unpermute<<<grid_for(n), 256, 0, (cudaStream_t)s>>>(a, out, f32, n, n1);
  return ok();
}
int aw_k_vdot(const void* a, const void* b, int f32, long long n, double2* part, int nblocks, void* s) {
  k_vdot<<<nblocks, 256, 0, (cudaStream_t)s>>>(a, b, f32, n, part);
  return ok();
}
int aw_k_axpy(void* y, const void* x, int f32, long long n, double cr, double ci, void* s) {
  k_axpy<<<grid_for(n), 256, 0, (cudaStream_t)s>>>(y, x, f32, n, cr, ci);
  return ok();
}
int aw_k_sum_parts(const double2* part, int nparts, int n, double2* out, void* s) {
  k_sum_parts<<<(n + 127) / 128, 128, 0, (cudaStream_t)s>>>(part, nparts, n, out);
  return ok();
}
int aw_k_set2(double* p, double a, double b, void* s) {
  k_set2<<<1, 1, 0, (cudaStream_t)s>>>(p, a, b);
  return ok();
}

}  // extern "C"
