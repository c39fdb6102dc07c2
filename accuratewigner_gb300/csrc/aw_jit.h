// Source of the user-expression module compiled at run time with NVRTC.
//
// The reference builds its kernels by str.format()-ing the user's strings
// (V, K, abs_boundary_*, observables, initial conditions) into CUDA-C
// templates and compiling them with PyCUDA's SourceModule
// (wigner_moyal_cuda_1d.py:241-247, :335-342, :400-406).  Here only the small
// kernels that evaluate those strings are generated: 1-D phase tables, 2-D
// absorbing masks, initial conditions, observable sums.  The FFT passes that
// consume the tables are compiled ahead of time (aw_pass.cuh).
//
// The user's strings see the same names as in the reference: the #define
// constants, `t`, the coordinates of the kernel they were written for, the
// indices i and j, cuda_complex and M_PI.  Every identifier the generated code
// adds carries an aw_ prefix so that a user #define cannot capture it.
#pragma once
#include <string>
#include <vector>

namespace awjit {

inline const char* prelude() {
  return R"AWSRC(
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
typedef unsigned long long aw_size_t;
struct cuda_complex {
  double _aw_re, _aw_im;
  __device__ cuda_complex() : _aw_re(0.0), _aw_im(0.0) {}
  __device__ cuda_complex(double r, double i = 0.0) : _aw_re(r), _aw_im(i) {}
  __device__ double real() const { return _aw_re; }
  __device__ double imag() const { return _aw_im; }
  __device__ cuda_complex& operator+=(const cuda_complex& o) { _aw_re += o._aw_re; _aw_im += o._aw_im; return *this; }
  __device__ cuda_complex& operator-=(const cuda_complex& o) { _aw_re -= o._aw_re; _aw_im -= o._aw_im; return *this; }
  __device__ cuda_complex& operator*=(const cuda_complex& o) {
    double r = _aw_re * o._aw_re - _aw_im * o._aw_im;
    _aw_im = _aw_re * o._aw_im + _aw_im * o._aw_re; _aw_re = r; return *this; }
  __device__ cuda_complex& operator/=(const cuda_complex& o) {
    double d = o._aw_re * o._aw_re + o._aw_im * o._aw_im;
    double r = (_aw_re * o._aw_re + _aw_im * o._aw_im) / d;
    _aw_im = (_aw_im * o._aw_re - _aw_re * o._aw_im) / d; _aw_re = r; return *this; }
};
__device__ inline cuda_complex operator+(cuda_complex a, const cuda_complex& b) { return a += b; }
__device__ inline cuda_complex operator-(cuda_complex a, const cuda_complex& b) { return a -= b; }
__device__ inline cuda_complex operator*(cuda_complex a, const cuda_complex& b) { return a *= b; }
__device__ inline cuda_complex operator/(cuda_complex a, const cuda_complex& b) { return a /= b; }
__device__ inline cuda_complex operator-(const cuda_complex& a) { return cuda_complex(-a._aw_re, -a._aw_im); }
__device__ inline cuda_complex operator+(const cuda_complex& a) { return a; }
__device__ inline double real(const cuda_complex& a) { return a._aw_re; }
__device__ inline double imag(const cuda_complex& a) { return a._aw_im; }
__device__ inline cuda_complex conj(const cuda_complex& a) { return cuda_complex(a._aw_re, -a._aw_im); }
__device__ inline double abs(const cuda_complex& a) { return hypot(a._aw_re, a._aw_im); }
__device__ inline double arg(const cuda_complex& a) { return atan2(a._aw_im, a._aw_re); }
__device__ inline double norm(const cuda_complex& a) { return a._aw_re * a._aw_re + a._aw_im * a._aw_im; }
__device__ inline cuda_complex exp(const cuda_complex& a) {
  double e = exp(a._aw_re), s, c; sincos(a._aw_im, &s, &c); return cuda_complex(e * c, e * s); }
__device__ inline cuda_complex log(const cuda_complex& a) { return cuda_complex(log(abs(a)), arg(a)); }
__device__ inline cuda_complex pow(const cuda_complex& a, double p) {
  if (a._aw_re == 0.0 && a._aw_im == 0.0) return cuda_complex(0.0, 0.0);
  return exp(cuda_complex(p, 0.0) * log(a)); }
__device__ inline cuda_complex pow(const cuda_complex& a, int p) { return pow(a, (double)p); }
__device__ inline cuda_complex pow(const cuda_complex& a, const cuda_complex& p) {
  if (a._aw_re == 0.0 && a._aw_im == 0.0) return cuda_complex(0.0, 0.0);
  return exp(p * log(a)); }
__device__ inline cuda_complex pow(double a, const cuda_complex& p) { return exp(p * cuda_complex(log(a), 0.0)); }
__device__ inline cuda_complex sqrt(const cuda_complex& a) { return pow(a, 0.5); }
template <typename T> __device__ inline void aw_store(void* aw_p, long long aw_k, int aw_f32, T aw_v);
template <> __device__ inline void aw_store<double>(void* aw_p, long long aw_k, int aw_f32, double aw_v) {
  if (aw_f32) ((float2*)aw_p)[aw_k] = make_float2((float)aw_v, 0.f);
  else ((double2*)aw_p)[aw_k] = make_double2(aw_v, 0.0); }
template <> __device__ inline void aw_store<cuda_complex>(void* aw_p, long long aw_k, int aw_f32, cuda_complex aw_v) {
  if (aw_f32) ((float2*)aw_p)[aw_k] = make_float2((float)aw_v._aw_re, (float)aw_v._aw_im);
  else ((double2*)aw_p)[aw_k] = make_double2(aw_v._aw_re, aw_v._aw_im); }
// double-float form of a table entry (format 2): each FP64 number as the FP32 pair (hi, lo); a
// complex entry as (re hi, im hi, re lo, im lo)
__device__ inline float2 aw_df1(double aw_v) {
  const float aw_h = (float)aw_v;
  return make_float2(aw_h, (float)(aw_v - (double)aw_h));
}
__device__ inline float4 aw_df2(double aw_re, double aw_im) {
  const float2 aw_a = aw_df1(aw_re), aw_b = aw_df1(aw_im);
  return make_float4(aw_a.x, aw_b.x, aw_a.y, aw_b.y);
}
__device__ inline double2 aw_load(const void* aw_p, long long aw_k, int aw_f32) {
  if (aw_f32) { float2 aw_v = ((const float2*)aw_p)[aw_k]; return make_double2(aw_v.x, aw_v.y); }
  return ((const double2*)aw_p)[aw_k]; }
// block sum for blocks of whole warps: a fixed shuffle tree in each warp, then every thread adds the
// warp sums in index order (the same value in every thread)
__device__ inline double aw_block_sum(double aw_v, double* aw_red) {
  const int aw_t = threadIdx.x;
  for (int aw_o = 16; aw_o > 0; aw_o >>= 1) aw_v += __shfl_down_sync(0xffffffffu, aw_v, aw_o);
  if ((aw_t & 31) == 0) aw_red[aw_t >> 5] = aw_v;
  __syncthreads();
  double aw_r = 0.0;
  for (int aw_w = 0; aw_w < (int)(blockDim.x >> 5); ++aw_w) aw_r += aw_red[aw_w];
  __syncthreads();
  return aw_r;
}
)AWSRC";
}

// coordinate names of each propagator kind, as the reference's kernels declare them
struct KindNames {
  bool rotated;     // WM/WB: (XX, XX_prime) and (PP, PP_prime) grids, 2-D masks
  bool vn;          // VN/RB: abs_boundary_x(X), abs_boundary_p(P) functions
  bool sw;          // SW: 1-D wave function
};

// Per-instance parameters (batched propagators): each name becomes a macro that reads the
// instance's row of the parameter table, through the aw_prm argument that every function of a
// user expression takes (null for a single propagator, whose constants are #defines).
inline std::string param_macros(const std::vector<std::string>& params) {
  std::string s;
  for (size_t k = 0; k < params.size(); ++k)
    s += "#define " + params[k] + " (aw_prm[" + std::to_string(k) + "])\n";
  return s;
}

inline std::string module_source(const KindNames& kn, const std::string& consts, const std::string& V,
                                 const std::string& K, const std::string& absx, const std::string& absp,
                                 const std::vector<std::string>& obs_x, const std::vector<std::string>& obs_p,
                                 const std::vector<std::string>& params = {}, const std::string& init = "") {
  std::string s = prelude();
  s += "\n// ---- user constants and functions\n";
  s += consts;
  s += "\n";
  s += param_macros(params);
  s += "\n// ---- energies (wigner_moyal_cuda_1d.py:723-733)\n";
  s += "__device__ double K(double P, double t, const double* aw_prm) { return (" + K + "); }\n";
  s += "__device__ double V(double X, double t, const double* aw_prm) { return (" + V + "); }\n";
  if (kn.rotated) {
    s += "__device__ double aw_absx2d(aw_size_t i, aw_size_t j, double XX, double XX_prime, double PP, double PP_prime, double t, const double* aw_prm) { return (" + absx + "); }\n";
    s += "__device__ double aw_absp2d(aw_size_t i, aw_size_t j, double XX, double XX_prime, double PP, double PP_prime, double t, const double* aw_prm) { return (" + absp + "); }\n";
    s += "__device__ double aw_mask1(int aw_fn, aw_size_t j, double aw_x, double t, const double* aw_prm) { return 1.0; }\n";
  } else if (kn.vn) {
    s += "__device__ double abs_boundary_x(double X, const double* aw_prm) { return (" + absx + "); }\n";
    s += "__device__ double abs_boundary_p(double P, const double* aw_prm) { return (" + absp + "); }\n";
    s += "__device__ double aw_mask1(int aw_fn, aw_size_t j, double aw_x, double t, const double* aw_prm) { return aw_fn == 0 ? abs_boundary_x(aw_x, aw_prm) : abs_boundary_p(aw_x, aw_prm); }\n";
  } else {
    s += "__device__ double aw_absx1(aw_size_t j, double X, double t, const double* aw_prm) { return (" + absx + "); }\n";
    s += "__device__ double aw_absp1(aw_size_t j, double P, double t, const double* aw_prm) { return (" + absp + "); }\n";
    s += "__device__ double aw_mask1(int aw_fn, aw_size_t j, double aw_x, double t, const double* aw_prm) { return aw_fn == 0 ? aw_absx1(j, aw_x, t, aw_prm) : aw_absp1(j, aw_x, t, aw_prm); }\n";
  }
  s += "__device__ double aw_obs_x(int aw_k, double X, double t, const double* aw_prm) {\n  switch (aw_k) {\n";
  for (size_t k = 0; k < obs_x.size(); ++k) s += "    case " + std::to_string(k) + ": return (" + obs_x[k] + ");\n";
  s += "  }\n  return 0.0;\n}\n";
  s += "__device__ double aw_obs_p(int aw_k, double P, double t, const double* aw_prm) {\n  switch (aw_k) {\n";
  for (size_t k = 0; k < obs_p.size(); ++k) s += "    case " + std::to_string(k) + ": return (" + obs_p[k] + ");\n";
  s += "  }\n  return 0.0;\n}\n";
  if (!init.empty()) {
    // initial state of one instance of a batch: W(X, P) for the rotated frame, rho(X, X_prime) else
    if (kn.rotated)
      s += "__device__ cuda_complex aw_init_value(aw_size_t i, aw_size_t j, double X, double P, const double* aw_prm) { return cuda_complex(" + init + "); }\n";
    else
      s += "__device__ cuda_complex aw_init_value(aw_size_t i, aw_size_t j, double X, double X_prime, const double* aw_prm) { return cuda_complex(" + init + "); }\n";
    s += R"AWSRC(
extern "C" __global__ void aw_binit(void* aw_out, int aw_f32, int aw_nrow, int aw_ncol, double aw_dX, double aw_dP,
                                    const double* aw_prm) {
  const aw_size_t i = blockIdx.y;
  const aw_size_t j = (aw_size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= (aw_size_t)aw_ncol) return;
  const double aw_a = aw_dX * (j - 0.5 * aw_ncol);
  const double aw_b = aw_dP * (i - 0.5 * aw_nrow);
  aw_store(aw_out, (long long)i * aw_ncol + j, aw_f32, aw_init_value(i, j, aw_a, aw_b, aw_prm));
}
)AWSRC";
  }
  s += R"AWSRC(
// 1-D tables of phase factors.  Column entries (aw_ncol of them) sit on the
// grid x_j = aw_dcol (((j + aw_roll) mod aw_ncol) - aw_ncol/2), row entries on
// x_i = aw_drow (i - aw_nrow/2).  aw_mode 0: exp(i (ca F(x,ta) + cb F(x,tb)));
// aw_mode 1: exp(ca (F(x,ta) - shift)) (real).  F = V (aw_fn 0) or K (aw_fn 1).
// aw_maskpow > 0 multiplies by the one-dimensional absorbing boundary.
// With aw_tlist, blockIdx.y = s builds the tables of time aw_tlist[s] + aw_ta at
// aw_col / aw_row + s * aw_tstride elements (one launch for a run of time points).
// Batches: blockIdx.z = instance, whose tables sit aw_istride elements apart, with its own
// parameters (aw_params + instance * aw_np) and, when given, its own aw_ca / aw_shift.
extern "C" __global__ void aw_tab(void* aw_col, void* aw_row, int aw_f32, int aw_fn, int aw_mode,
                                  int aw_ncol, double aw_dcol, int aw_roll, int aw_nrow, double aw_drow,
                                  double aw_ta, double aw_tb, double aw_ca, double aw_cb, double aw_shift,
                                  int aw_maskpow, double aw_tmask, const double* aw_tlist, long long aw_tstride,
                                  const double* aw_params, int aw_np, const double* aw_ca_vec,
                                  const double* aw_shift_vec, long long aw_istride) {
  const int aw_k = blockIdx.x * blockDim.x + threadIdx.x;
  if (aw_k >= aw_ncol + aw_nrow) return;
  const int aw_inst = blockIdx.z;
  const double* aw_prm = aw_params ? aw_params + (long long)aw_inst * aw_np : nullptr;
  if (aw_ca_vec) aw_ca = aw_ca_vec[aw_inst];
  if (aw_shift_vec) aw_shift = aw_shift_vec[aw_inst];
  const int aw_esz = aw_f32 == 1 ? 8 : 16;
  long long aw_off = aw_inst * aw_istride * aw_esz;
  if (aw_tlist) {
    const int aw_s = blockIdx.y;
    aw_ta += aw_tlist[aw_s];
    aw_off += aw_s * aw_tstride * aw_esz;
  }
  aw_col = (char*)aw_col + aw_off;
  aw_row = (char*)aw_row + aw_off;
  const bool aw_c = aw_k < aw_ncol;
  const int aw_n = aw_c ? aw_ncol : aw_nrow;
  const int aw_idx = aw_c ? aw_k : aw_k - aw_ncol;
  const aw_size_t aw_m = aw_c ? (aw_size_t)((aw_idx + aw_roll) % aw_n) : (aw_size_t)aw_idx;
  const double aw_x = (aw_c ? aw_dcol : aw_drow) * (aw_m - 0.5 * aw_n);
  double aw_re, aw_im;
  if (aw_mode == 0) {
    double aw_ph = aw_ca * (aw_fn == 0 ? V(aw_x, aw_ta, aw_prm) : K(aw_x, aw_ta, aw_prm));
    if (aw_cb != 0.0) aw_ph += aw_cb * (aw_fn == 0 ? V(aw_x, aw_tb, aw_prm) : K(aw_x, aw_tb, aw_prm));
    sincos(aw_ph, &aw_im, &aw_re);
  } else {
    aw_re = exp(aw_ca * ((aw_fn == 0 ? V(aw_x, aw_ta, aw_prm) : K(aw_x, aw_ta, aw_prm)) - aw_shift));
    aw_im = 0.0;
  }
  if (aw_maskpow > 0) {
    double aw_q = aw_mask1(aw_fn, aw_m, aw_x, aw_tmask, aw_prm);
    double aw_f = aw_maskpow == 2 ? aw_q * aw_q : aw_q;
    aw_re *= aw_f;
    aw_im *= aw_f;
  }
  void* aw_dst = aw_c ? aw_col : aw_row;
  if (aw_f32 == 1) ((float2*)aw_dst)[aw_idx] = make_float2((float)aw_re, (float)aw_im);
  else if (aw_f32 == 2) ((float4*)aw_dst)[aw_idx] = aw_df2(aw_re, aw_im);
  else ((double2*)aw_dst)[aw_idx] = make_double2(aw_re, aw_im);
}

// Plain values of V or K on a 1-D grid (Bloch minima, rho_bloch/wigner_bloch fill kernels).
// blockIdx.y = instance of a batch: output row aw_ostride apart, its own parameters
extern "C" __global__ void aw_values(double* aw_out, int aw_fn, int aw_n, double aw_d, double aw_t,
                                     const double* aw_params, int aw_np, long long aw_ostride) {
  const int aw_k = blockIdx.x * blockDim.x + threadIdx.x;
  if (aw_k >= aw_n) return;
  const int aw_inst = blockIdx.y;
  const double* aw_prm = aw_params ? aw_params + (long long)aw_inst * aw_np : nullptr;
  const double aw_x = aw_d * ((aw_size_t)aw_k - 0.5 * aw_n);
  aw_out[aw_inst * aw_ostride + aw_k] = aw_fn == 0 ? V(aw_x, aw_t, aw_prm) : K(aw_x, aw_t, aw_prm);
}

// Per-step observables from the marginals of the state.
//   aw_colsum[j * aw_cstride]: X-marginal on x_j = dX (j - ncol/2)
//   aw_rowpart[p][i] (p < aw_nparts): partial P-marginals on p_i = dP (((i + aw_proll) mod nrow) - nrow/2)
// For the rotated frame these are the column and row sums of Re W; for the
// density matrix the diagonal in x and in p; for the wave function |psi|^2
// and |fft psi|^2.  Slots are sums of X-only / P-only averages normalised by
// norm = Sum colsum * aw_dXdP (P-terms by their own marginal when
// aw_pnorm_own), as wigner_moyal_cuda_1d.py:608-622 normalises W.  The kernel
// also writes the purity 2 pi Sum W^2 dXdP / norm^2 (rotated frame), the norm,
// and the factor the next pass applies: 1 / norm (or 1 / sqrt(norm) when
// aw_sqrt_norm, for a wave function), and the P-marginal aw_rowsum.
// Blocks: (term, X norm, P norm, sum of squares) x chunk of columns or rows, so that the FP64
// expression work spreads over the SMs (one block took 138 us for the 4096-point von Neumann
// observables); each block's partial goes to aw_tv, and the last block to finish adds them in a fixed
// order.
extern "C" __global__ void aw_finalize(const double* aw_colsum, const double* aw_rowpart, int aw_nparts,
                                       const double* aw_sqpart, double* aw_rowsum, double* aw_hist,
                                       double* aw_inv_norm, int* aw_stop, int aw_stop_on_purity, double t,
                                       int aw_ncol, int aw_nrow, double aw_dX, double aw_dP, double aw_dXdP,
                                       const int* aw_tslot, const int* aw_tkind, const int* aw_tidx,
                                       const double* aw_tcoef, int aw_nterms, int aw_nslots,
                                       int aw_cstride, int aw_proll, int aw_pnorm_own, int aw_sqrt_norm,
                                       const double* aw_prm, double* aw_tv, unsigned int* aw_counter, int aw_nchunk) {
  __shared__ double aw_red[256];
  __shared__ double aw_fsum[67];
  __shared__ double aw_scoef[64];
  __shared__ int aw_sslot[64], aw_skind[64];
  __shared__ int aw_is_last;
  if (aw_stop && *aw_stop) return;
  const int aw_q = blockIdx.x / aw_nchunk;  // < nterms: a term; nterms: X norm; +1: P norm; +2: squares
  const int aw_c = blockIdx.x - aw_q * aw_nchunk;
  const int aw_t = threadIdx.x;
  const int aw_nt = blockDim.x;
  const bool aw_on_rows = (aw_q < aw_nterms && aw_tkind[aw_q] != 0) || aw_q == aw_nterms + 1;
  const int aw_n = aw_on_rows ? aw_nrow : aw_ncol;
  const int aw_len = (aw_n + aw_nchunk - 1) / aw_nchunk;
  const int aw_lo = aw_c * aw_len;
  const int aw_hi = aw_lo + aw_len < aw_n ? aw_lo + aw_len : aw_n;
  double aw_s = 0.0;
  if (aw_q < aw_nterms) {
    const int aw_idx = aw_tidx[aw_q];
    if (!aw_on_rows) {
      for (int aw_j = aw_lo + aw_t; aw_j < aw_hi; aw_j += aw_nt) {
        const double X = aw_dX * ((aw_size_t)aw_j - 0.5 * aw_ncol);
        aw_s += aw_colsum[(long long)aw_j * aw_cstride] * aw_obs_x(aw_idx, X, t, aw_prm);
      }
    } else {
      for (int aw_i = aw_lo + aw_t; aw_i < aw_hi; aw_i += aw_nt) {
        double aw_r = 0.0;
        for (int aw_p = 0; aw_p < aw_nparts; ++aw_p) aw_r += aw_rowpart[(long long)aw_p * aw_nrow + aw_i];
        const double P = aw_dP * ((aw_size_t)((aw_i + aw_proll) % aw_nrow) - 0.5 * aw_nrow);
        aw_s += aw_r * aw_obs_p(aw_idx, P, t, aw_prm);
      }
    }
  } else if (aw_q == aw_nterms) {
    for (int aw_j = aw_lo + aw_t; aw_j < aw_hi; aw_j += aw_nt) aw_s += aw_colsum[(long long)aw_j * aw_cstride];
  } else if (aw_q == aw_nterms + 1) {
    for (int aw_i = aw_lo + aw_t; aw_i < aw_hi; aw_i += aw_nt) {
      double aw_r = 0.0;
      for (int aw_p = 0; aw_p < aw_nparts; ++aw_p) aw_r += aw_rowpart[(long long)aw_p * aw_nrow + aw_i];
      aw_rowsum[aw_i] = aw_r;
      aw_s += aw_r;
    }
  } else if (aw_sqpart) {
    for (int aw_p = aw_c * aw_nt + aw_t; aw_p < aw_nparts; aw_p += aw_nt * aw_nchunk) aw_s += aw_sqpart[aw_p];
  }
  const double aw_v = aw_block_sum(aw_s, aw_red);
  if (aw_t == 0) {
    aw_tv[blockIdx.x] = aw_v;
    __threadfence();
    const unsigned int aw_prev = atomicAdd(aw_counter, 1u);
    aw_is_last = aw_prev == gridDim.x - 1;
  }
  __syncthreads();
  if (!aw_is_last) return;
  __threadfence();
  // the terms' slots, kinds and coefficients, staged for the per-slot sums below
  for (int aw_k = aw_t; aw_k < aw_nterms; aw_k += aw_nt) {
    aw_sslot[aw_k] = aw_tslot[aw_k];
    aw_skind[aw_k] = aw_tkind[aw_k];
    aw_scoef[aw_k] = aw_tcoef[aw_k];
  }
  // one warp per term (or norm, or squares): lanes sum over the chunks, then a shuffle tree
  const volatile double* aw_vt = aw_tv;
  const int aw_lane = aw_t & 31;
  for (int aw_k = aw_t >> 5; aw_k < aw_nterms + 3; aw_k += aw_nt >> 5) {
    double aw_acc = 0.0;
    for (int aw_cc = aw_lane; aw_cc < aw_nchunk; aw_cc += 32) aw_acc += aw_vt[aw_k * aw_nchunk + aw_cc];
    for (int aw_o = 16; aw_o > 0; aw_o >>= 1) aw_acc += __shfl_down_sync(0xffffffffu, aw_acc, aw_o);
    if (aw_lane == 0) aw_fsum[aw_k] = aw_acc;
  }
  __syncthreads();
  const double aw_norm = aw_fsum[aw_nterms] * aw_dXdP;
  const double aw_pnorm_raw = aw_fsum[aw_nterms + 1];
  // each slot by its own thread: its terms added in term order from zero, the sums one thread's loop
  // over the terms into a zeroed row makes, without that loop's chain of dependent global loads and
  // stores (it was most of this kernel's time on small grids)
  for (int aw_s2 = aw_t; aw_s2 < aw_nslots; aw_s2 += aw_nt) {
    double aw_h = 0.0;
    for (int aw_k = 0; aw_k < aw_nterms; ++aw_k) {
      if (aw_sslot[aw_k] != aw_s2) continue;
      const bool aw_own = aw_pnorm_own && aw_skind[aw_k] == 1;
      aw_h += aw_scoef[aw_k] * (aw_own ? aw_fsum[aw_k] / aw_pnorm_raw : aw_fsum[aw_k] * aw_dXdP / aw_norm);
    }
    aw_hist[aw_s2] = aw_h;
  }
  if (aw_t == 0) {
    const double aw_purity = 2.0 * M_PI * aw_fsum[aw_nterms + 2] * aw_dXdP / (aw_norm * aw_norm);
    aw_hist[aw_nslots] = aw_purity;
    aw_hist[aw_nslots + 1] = aw_norm;
    if (aw_inv_norm) {
      aw_inv_norm[0] = aw_sqrt_norm ? 1.0 / sqrt(aw_norm) : 1.0 / aw_norm;
      aw_inv_norm[1] = 0.0;
    }
    if (aw_stop && aw_stop_on_purity && !(aw_purity < 1.0)) *aw_stop = 1;
    *aw_counter = 0u;
  }
}
)AWSRC";
  if (kn.rotated) {
    s += R"AWSRC(
// Per-step observables of the rotated frame from one column FFT of the Wigner transform's first
// stage A (W = S ifft0 C ifft0 (shY . fft0 A), C = the second X shear; see rot_run in aw_api.cu).
// With Q_j = shY_j . fft0(A_j):
//   X-marginal  c_j = Sum_i Re W_ij = (-1)^j Np Re z_j,            z_j = Sum_m (-1)^m Q_j(m)
//   P-marginal  r_i = Sum_j Re W_ij = (-1)^i Np Re w_{(-i) mod Np},  w_m = Sum_j (-1)^j Q_j(m)
//   purity      2 pi dXdP Sum Re W^2 / norm^2 = 2 pi dXdP Np Sum |rho|^2 / norm^2 (the transform is
//               unitary up to the factor Np of the unnormalised ifft0)
// Blocks per term, for the norm and for Sum |rho|^2, each over a chunk of columns or rows; the last
// block to finish combines them in a fixed order.
extern "C" __global__ void aw_finalize_rot(const double2* aw_z, const double2* aw_wpart, int aw_nparts,
                                           const double* aw_abs2, int aw_nb2, double* aw_tv, unsigned int* aw_counter,
                                           double* aw_hist, double* aw_inv_norm, int* aw_stop, int aw_stop_on_purity,
                                           double aw_t_arg, int aw_ncol, int aw_nrow, double aw_dX, double aw_dP,
                                           double aw_dXdP, const int* aw_tslot, const int* aw_tkind,
                                           const int* aw_tidx, const double* aw_tcoef, int aw_nterms, int aw_nslots,
                                           int aw_nchunk, const double* aw_params, int aw_np, long long aw_hstride,
                                           const double* aw_tptr) {
  // blocks: (term or norm or purity) x chunk; FP64 expression evaluation spread over the GPU.
  // blockIdx.y = instance of a batch, with its own marginals, partials, history row and scalars.
  // The observables' time: the argument, or (a step loop replayed from a CUDA graph) read from aw_tptr.
  const double t = aw_tptr ? *aw_tptr : aw_t_arg;
  __shared__ double aw_red[256];
  __shared__ double aw_wg[256];
  __shared__ double aw_fsum[66];
  __shared__ double aw_scoef[64];
  __shared__ int aw_sslot[64];
  __shared__ int aw_is_last;
  {
    const long long aw_in = blockIdx.y;
    aw_z += aw_in * aw_ncol;
    aw_wpart += aw_in * aw_nparts * aw_nrow;
    if (aw_abs2) aw_abs2 += aw_in * aw_nb2;
    aw_tv += aw_in * gridDim.x;
    aw_counter += aw_in;
    aw_hist += aw_in * aw_hstride;
    aw_inv_norm += 2 * aw_in;
    if (aw_stop) aw_stop += aw_in;
  }
  const double* aw_prm = aw_params ? aw_params + (long long)blockIdx.y * aw_np : nullptr;
  if (aw_stop && *aw_stop) return;
  const int aw_q = blockIdx.x / aw_nchunk;      // 0..nterms-1 terms, nterms norm, nterms+1 purity
  const int aw_c = blockIdx.x - aw_q * aw_nchunk;
  const int aw_t = threadIdx.x;
  const int aw_nt = blockDim.x;
  double aw_s = 0.0;
  if (aw_q < aw_nterms) {
    const int aw_idx = aw_tidx[aw_q];
    if (aw_tkind[aw_q] == 0) {
      const int aw_len = aw_ncol / aw_nchunk, aw_lo = aw_c * aw_len;
      for (int aw_j = aw_lo + aw_t; aw_j < aw_lo + aw_len; aw_j += aw_nt) {
        const double X = aw_dX * ((aw_size_t)aw_j - 0.5 * aw_ncol);
        const double aw_cj = ((aw_j & 1) ? -1.0 : 1.0) * aw_nrow * aw_z[aw_j].x;
        aw_s += aw_cj * aw_obs_x(aw_idx, X, t, aw_prm);
      }
    } else {
      // aw_gs threads share each row's partials (every aw_gs-th one, in four interleaved sums so that
      // their loads are in flight together); the group sums meet in shared memory and add in a fixed
      // order.  Row counts and the block size are powers of two, so every sweep fills the block.
      const int aw_len = aw_nrow / aw_nchunk, aw_lo = aw_c * aw_len;
      const int aw_gs = aw_len < aw_nt ? aw_nt / aw_len : 1;
      const int aw_rows = aw_nt / aw_gs;
      const int aw_r = aw_t % aw_rows, aw_g = aw_t / aw_rows;
      for (int aw_i0 = aw_lo; aw_i0 < aw_lo + aw_len; aw_i0 += aw_rows) {
        const int aw_i = aw_i0 + aw_r;
        const int aw_k = (aw_nrow - aw_i) & (aw_nrow - 1);
        double aw_w0 = 0.0, aw_w1 = 0.0, aw_w2 = 0.0, aw_w3 = 0.0;
        int aw_p = aw_g;
        for (; aw_p + 3 * aw_gs < aw_nparts; aw_p += 4 * aw_gs) {
          aw_w0 += aw_wpart[(long long)aw_p * aw_nrow + aw_k].x;
          aw_w1 += aw_wpart[(long long)(aw_p + aw_gs) * aw_nrow + aw_k].x;
          aw_w2 += aw_wpart[(long long)(aw_p + 2 * aw_gs) * aw_nrow + aw_k].x;
          aw_w3 += aw_wpart[(long long)(aw_p + 3 * aw_gs) * aw_nrow + aw_k].x;
        }
        for (; aw_p < aw_nparts; aw_p += aw_gs) aw_w0 += aw_wpart[(long long)aw_p * aw_nrow + aw_k].x;
        aw_wg[aw_t] = (aw_w0 + aw_w1) + (aw_w2 + aw_w3);
        __syncthreads();
        if (aw_g == 0) {
          double aw_w = aw_wg[aw_r];
          for (int aw_q2 = 1; aw_q2 < aw_gs; ++aw_q2) aw_w += aw_wg[aw_q2 * aw_rows + aw_r];
          const double P = aw_dP * ((aw_size_t)aw_i - 0.5 * aw_nrow);
          aw_s += ((aw_i & 1) ? -1.0 : 1.0) * aw_nrow * aw_w * aw_obs_p(aw_idx, P, t, aw_prm);
        }
        __syncthreads();
      }
    }
  } else if (aw_q == aw_nterms) {
    const int aw_len = aw_ncol / aw_nchunk, aw_lo = aw_c * aw_len;
    for (int aw_j = aw_lo + aw_t; aw_j < aw_lo + aw_len; aw_j += aw_nt)
      aw_s += ((aw_j & 1) ? -1.0 : 1.0) * aw_nrow * aw_z[aw_j].x;
  } else if (aw_abs2) {
    for (int aw_p = aw_c * aw_nt + aw_t; aw_p < aw_nb2; aw_p += aw_nt * aw_nchunk) aw_s += aw_abs2[aw_p];
  }
  const double aw_v = aw_block_sum(aw_s, aw_red);
  if (aw_t == 0) {
    aw_tv[blockIdx.x] = aw_v;
    __threadfence();
    const unsigned int aw_prev = atomicAdd(aw_counter, 1u);
    aw_is_last = aw_prev == gridDim.x - 1;
  }
  __syncthreads();
  if (aw_is_last) {
    __threadfence();
    // the terms' slots and coefficients, staged for the per-slot sums below
    for (int aw_k = aw_t; aw_k < aw_nterms; aw_k += aw_nt) {
      aw_sslot[aw_k] = aw_tslot[aw_k];
      aw_scoef[aw_k] = aw_tcoef[aw_k];
    }
    // one warp per term (or norm, or purity): lane sums over the chunks, then a shuffle tree
    const volatile double* aw_vt = aw_tv;
    const int aw_lane = aw_t & 31;
    for (int aw_k = aw_t >> 5; aw_k < aw_nterms + 2; aw_k += aw_nt >> 5) {
      double aw_acc = 0.0;
      for (int aw_cc = aw_lane; aw_cc < aw_nchunk; aw_cc += 32) aw_acc += aw_vt[aw_k * aw_nchunk + aw_cc];
      for (int aw_o = 16; aw_o > 0; aw_o >>= 1) aw_acc += __shfl_down_sync(0xffffffffu, aw_acc, aw_o);
      if (aw_lane == 0) aw_fsum[aw_k] = aw_acc;
    }
    __syncthreads();
    const double* aw_sum = aw_fsum;
    const double aw_norm = aw_sum[aw_nterms] * aw_dXdP;
    // each slot by its own thread: its terms added in term order from zero, the sums one thread's
    // loop over the terms into a zeroed row makes, without that loop's chain of dependent global
    // loads and stores (it was most of this kernel's time on small grids)
    for (int aw_s2 = aw_t; aw_s2 < aw_nslots; aw_s2 += aw_nt) {
      double aw_h = 0.0;
      for (int aw_k = 0; aw_k < aw_nterms; ++aw_k)
        if (aw_sslot[aw_k] == aw_s2) aw_h += aw_scoef[aw_k] * (aw_sum[aw_k] * aw_dXdP / aw_norm);
      aw_hist[aw_s2] = aw_h;
    }
    if (aw_t == 0) {
      const double aw_purity = 2.0 * M_PI * aw_dXdP * aw_nrow * aw_sum[aw_nterms + 1] / (aw_norm * aw_norm);
      aw_hist[aw_nslots] = aw_purity;
      aw_hist[aw_nslots + 1] = aw_norm;
      aw_inv_norm[0] = 1.0 / aw_norm;
      aw_inv_norm[1] = 0.0;
      if (aw_stop && aw_stop_on_purity && !(aw_purity < 1.0)) *aw_stop = 1;
      *aw_counter = 0u;
    }
  }
}

// 2-D absorbing boundaries of the rotated frame (expV / expK of
// wigner_moyal_cuda_1d.py:742-778 multiply by these expressions).
// blockIdx.z = instance of a batch: mask aw_nrow * aw_ncol elements apart, its own parameters
extern "C" __global__ void aw_mask2d(void* aw_out, int aw_f32, int aw_which, double t, int aw_nrow, int aw_ncol,
                                     double aw_dXX, double aw_dXXp, double aw_dPP, double aw_dPPp,
                                     const double* aw_params, int aw_np) {
  const aw_size_t i = blockIdx.y;
  const double* aw_prm = aw_params ? aw_params + (long long)blockIdx.z * aw_np : nullptr;
  aw_out = (char*)aw_out + (long long)blockIdx.z * aw_nrow * aw_ncol * (aw_f32 == 1 ? 4 : 8);
  const aw_size_t j = (aw_size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= (aw_size_t)aw_ncol) return;
  const double XX = aw_dXX * (j - 0.5 * aw_ncol);
  const double XX_prime = aw_dXXp * (i - 0.5 * aw_nrow);
  const double PP = aw_dPP * (j - 0.5 * aw_ncol);
  const double PP_prime = aw_dPPp * (i - 0.5 * aw_nrow);
  const double aw_v = aw_which == 0 ? aw_absx2d(i, j, XX, XX_prime, PP, PP_prime, t, aw_prm)
                                    : aw_absp2d(i, j, XX, XX_prime, PP, PP_prime, t, aw_prm);
  const long long aw_k = (long long)i * aw_ncol + j;
  if (aw_f32 == 1) ((float*)aw_out)[aw_k] = (float)aw_v;
  else if (aw_f32 == 2) ((float2*)aw_out)[aw_k] = aw_df1(aw_v);
  else ((double*)aw_out)[aw_k] = aw_v;
}
)AWSRC";
  }
  return s;
}

// Initial condition module (one per expression string).
inline std::string init_source(const KindNames& kn, const std::string& consts, const std::string& expr) {
  std::string s = prelude();
  s += consts;
  s += "\n";
  if (kn.rotated) {
    // wigner_moyal_cuda_1d.py:791-801
    s += "extern \"C\" __global__ void aw_init(void* aw_out, int aw_f32, int aw_nrow, int aw_ncol, double aw_dX, double aw_dP) {\n"
         "  const aw_size_t i = blockIdx.y;\n"
         "  const aw_size_t j = (aw_size_t)blockIdx.x * blockDim.x + threadIdx.x;\n"
         "  if (j >= (aw_size_t)aw_ncol) return;\n"
         "  const double X = aw_dX * (j - 0.5 * aw_ncol);\n"
         "  const double P = aw_dP * (i - 0.5 * aw_nrow);\n"
         "  aw_store(aw_out, (long long)i * aw_ncol + j, aw_f32, (" + expr + "));\n}\n";
  } else if (kn.vn) {
    // rho_vneumann_cuda_1d.py:783-793
    s += "extern \"C\" __global__ void aw_init(void* aw_out, int aw_f32, int aw_nrow, int aw_ncol, double aw_dX, double aw_dP) {\n"
         "  const aw_size_t i = blockIdx.y;\n"
         "  const aw_size_t j = (aw_size_t)blockIdx.x * blockDim.x + threadIdx.x;\n"
         "  if (j >= (aw_size_t)aw_ncol) return;\n"
         "  const double X = aw_dX * (j - 0.5 * aw_ncol);\n"
         "  const double X_prime = aw_dX * (i - 0.5 * aw_nrow);\n"
         "  aw_store(aw_out, (long long)i * aw_ncol + j, aw_f32, (" + expr + "));\n}\n";
  } else {
    // schrodinger_wigner_cuda_1d.py:867-874
    s += "extern \"C\" __global__ void aw_init(void* aw_out, int aw_f32, int aw_nrow, int aw_ncol, double aw_dX, double aw_dP) {\n"
         "  const aw_size_t j = (aw_size_t)blockIdx.x * blockDim.x + threadIdx.x;\n"
         "  if (j >= (aw_size_t)aw_ncol) return;\n"
         "  const double X = aw_dX * (j - 0.5 * aw_ncol);\n"
         "  aw_store(aw_out, (long long)j, aw_f32, (" + expr + "));\n}\n";
  }
  return s;
}

// Observable module (one per expression string).
//   rotated: partial sums of Re W f(X, P, t) over the Wigner grid (wm:817-827)
//   vn:      rho[i][j] *= f(X, P, t), X and P both from column j (vn:811-821)
//   sw:      partial sums of |psi|^2 f(X, P, t), P fft-shifted (sw:893-901)
inline std::string observable_source(const KindNames& kn, const std::string& consts, const std::string& expr) {
  std::string s = prelude();
  s += consts;
  s += "\n";
  if (kn.rotated) {
    s += "extern \"C\" __global__ void aw_obs(const void* aw_W, int aw_f32, double t, double* aw_part, int aw_nrow, int aw_ncol, double aw_dX, double aw_dP) {\n"
         "  __shared__ double aw_red[256];\n"
         "  double aw_s = 0.0;\n"
         "  const long long aw_n = (long long)aw_nrow * aw_ncol;\n"
         "  for (long long aw_k = (long long)blockIdx.x * blockDim.x + threadIdx.x; aw_k < aw_n; aw_k += (long long)gridDim.x * blockDim.x) {\n"
         "    const aw_size_t i = aw_k / aw_ncol;\n"
         "    const aw_size_t j = aw_k - (long long)i * aw_ncol;\n"
         "    const double X = aw_dX * (j - 0.5 * aw_ncol);\n"
         "    const double P = aw_dP * (i - 0.5 * aw_nrow);\n"
         "    aw_s += aw_load(aw_W, aw_k, aw_f32).x * (" + expr + ");\n"
         "  }\n"
         "  aw_s = aw_block_sum(aw_s, aw_red);\n"
         "  if (threadIdx.x == 0) aw_part[blockIdx.x] = aw_s;\n}\n";
  } else if (kn.vn) {
    s += "extern \"C\" __global__ void aw_obs(void* aw_rho, int aw_f32, double t, double* aw_unused, int aw_nrow, int aw_ncol, double aw_dX, double aw_dP) {\n"
         "  const aw_size_t i = blockIdx.y;\n"
         "  const aw_size_t j = (aw_size_t)blockIdx.x * blockDim.x + threadIdx.x;\n"
         "  if (j >= (aw_size_t)aw_ncol) return;\n"
         "  const double P = aw_dP * (j - 0.5 * aw_ncol);\n"
         "  const double X = aw_dX * (j - 0.5 * aw_ncol);\n"
         "  const long long aw_k = (long long)i * aw_ncol + j;\n"
         "  double2 aw_v = aw_load(aw_rho, aw_k, aw_f32);\n"
         "  cuda_complex aw_r = cuda_complex(aw_v.x, aw_v.y) * cuda_complex(" + expr + ");\n"
         "  aw_store(aw_rho, aw_k, aw_f32, aw_r);\n}\n";
  } else {
    s += "extern \"C\" __global__ void aw_obs(const void* aw_psi, int aw_f32, double t, double* aw_part, int aw_nrow, int aw_ncol, double aw_dX, double aw_dP) {\n"
         "  __shared__ double aw_red[256];\n"
         "  double aw_s = 0.0;\n"
         "  for (long long aw_k = (long long)blockIdx.x * blockDim.x + threadIdx.x; aw_k < aw_ncol; aw_k += (long long)gridDim.x * blockDim.x) {\n"
         "    const aw_size_t j = aw_k;\n"
         "    const double X = aw_dX * (j - 0.5 * aw_ncol);\n"
         "    const double P = aw_dP * ((j + aw_ncol / 2) % aw_ncol - 0.5 * aw_ncol);\n"
         "    double2 aw_v = aw_load(aw_psi, aw_k, aw_f32);\n"
         "    aw_s += (aw_v.x * aw_v.x + aw_v.y * aw_v.y) * (" + expr + ");\n"
         "  }\n"
         "  aw_s = aw_block_sum(aw_s, aw_red);\n"
         "  if (threadIdx.x == 0) aw_part[blockIdx.x] = aw_s;\n}\n";
  }
  return s;
}

}  // namespace awjit
