// Launchers of the expression-free helper kernels (aw_util.cu).
#pragma once
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

int aw_k_scale(void* a, int f32, long long n, double re, double im, const double* ptr, void* s);
// complex128 shear factors of `lines` lines of npos positions from their hi x lo tables
int aw_k_shear_full(const void* hi, const void* lo, int lo_n, int lines, int npos, void* full, void* s);
// conj(row[i]) * (scale * col[j]) (complex128) at full[j * nr + i] (a column-pass factor as one table) or,
// with row_lines, at full[i * nc + j] (a row-pass factor)
int aw_k_sep_full(const void* col, const void* row, double scale, int nr, int nc, int row_lines, void* full, void* s);
// ninst instances of n elements, instance k scaled by ptr[2k..2k+1] (when ptr)
int aw_k_scale_n(void* a, int f32, long long n, int ninst, double re, double im, const double* ptr, void* s);
/* count tables of n complex entries, stride entries apart, each entry k times the real s[k] */
int aw_k_scale_lines(void* tab, int fmt, const double* s, int n, int count, long long stride, void* st);
int aw_k_fill(void* a, int f32, long long n, double re, double im, void* s);
int aw_k_convert(const void* src, int sf32, void* dst, int df32, long long n, void* s);
int aw_k_partial(const void* a, int f32, long long n, int mode, long long stride, double2* part, int nblocks, void* s);
int aw_k_embed(const void* rho, int f32, int N, void* W, int M, int pad, void* s);
int aw_k_psi2rho(const void* psi, int f32, int N, void* rho, void* s);
int aw_k_trace_finalize(const double2* diag, int n, const double* abs2part, int nparts, double dX, int complex_trace,
                        double* inv_out, double* hist, int* stop, int stop_on_purity, void* s);
int aw_k_trace_finalize_n(const double2* diag, int n, const double* abs2part, int nparts, double dX, int complex_trace,
                          double* inv_out, double* hist, long long hstride, int* stop, int stop_on_purity, int ninst,
                          void* s);
int aw_k_set2(double* p, double a, double b, void* s);
// Re M_k = scale Re Sum_d g_d exp(-2 pi i k d / n) for k < n (n a power of two; scratch: n complex)
int aw_k_diag_dft(const double2* g, int n, double2* scratch, double* out_re, double scale, void* s);
// 1 / trace of every instance of up to 8 propagators (the grouped von Neumann step), member by member
typedef struct AwTraceGroup {
  int count, complex_trace;
  const double2* diag[8];
  int n[8], ninst[8];
  double dX[8];
  double* inv[8];
  int* stop[8];
} AwTraceGroup;
int aw_k_trace_finalize_group(const AwTraceGroup* g, void* s);
int aw_k_sum_parts(const double2* part, int nparts, int n, double2* out, void* s);
int aw_k_norm_finalize(const double* parts, int nparts, double scale, double* inv_out, double* hist, void* s);
int aw_k_abs2(const void* a, int f32, long long n, double* out, void* s);
// |a|^2 of a spectrum held in the four-step order (k = k1 + n1 k2 at k1 (n / n1) + k2), in natural order
int aw_k_abs2_perm(const void* a, int f32, long long n, int n1, double* out, void* s);
// a four-step spectrum into natural order
int aw_k_unpermute(const void* a, void* out, int f32, long long n, int n1, void* s);
int aw_k_vdot(const void* a, const void* b, int f32, long long n, double2* part, int nblocks, void* s);
int aw_k_axpy(void* y, const void* x, int f32, long long n, double cr, double ci, void* s);

#ifdef __cplusplus
}
#endif
