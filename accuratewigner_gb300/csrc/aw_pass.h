// Argument blocks of the fused FFT pass kernels (host and device side).
//
// One pass reads a tile of whole lines (rows or columns of the grid) once,
// runs a short fixed program on it in shared memory and writes it once:
//
//   load -> f0 -> [FFT d1] -> f1 -> (branch point) -> f2 -> [FFT d2] -> f3 -> store/reduce
//                                       |
//                                       +-> [FFT br_d1] -> fbr -> [FFT br_d2] -> store br_out
//
// which covers every cuFFT-plus-elementwise sequence of the reference's steps
// (wigner_moyal_cuda_1d.py:543-561), Wigner transforms (:422-501) and Bloch
// steps (wigner_bloch_cuda_1d.py:221-240).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Per-element multiplier.  Every field is optional; the product of the active
// parts is applied:  scale * (*scale_ptr) * (-1)^(i+j) * col_tab[j]
//                     * conj(row_tab[i]) * mask[i][j]^mask_pow * shear(line, pos)
typedef struct AwFactor {
  const void* col_tab;      // complex, one per grid column j
  const void* row_tab;      // complex, one per grid row i (used conjugated)
  const void* mask;         // real, [nrows][ncols]
  const void* sh_hi;        // shear table, [lines][npos / sh_lo_n] complex
  const void* sh_lo;        // shear table, [lines][sh_lo_n] complex
  const void* sh_full;      // or the shear factors themselves, [lines][N] complex (replaces hi x lo)
  const double* scale_ptr;  // optional device scalar: complex (re, im), one per instance
  double scale;
  int mask_pow;             // 0: no mask
  int sign;                 // 1: multiply by (-1)^(i+j); 2: by (-1)^i; 3: by (-1)^j
  int sh_lo_n;              // 0: no shear
  int sh_roll;              // shear position index is (pos + sh_roll) mod npos
  int lin;                  // col_tab as one table over the grid read as a 1-D array: 1 at i * ncols + j
                            // (row-major order), 2 at i + nrows * j (the four-step FFT's spectrum order)
  int active;
} AwFactor;

typedef struct AwPassArgs {
  const void* in;
  void* out;                // may be 0 for a reduce-only pass
  int nrows, ncols;
  const void* tw;           // twiddle table of the transform length
  const void* twt_mq;       // native FP64: the tangent-form twiddle table of the transform length (aw_fft.cuh),
  const unsigned char* twt_e;  // ... (m, q) pairs and exponents; required by the FP64 passes
  AwFactor f0;
  int d1;                   // 0: none, +1: forward, -1: inverse (unnormalised)
  AwFactor f1;
  void* mid_out;            // optional store of the tile at the branch point
  int mid_sign;             // ... multiplied by (-1)^(i+j)
  void* br_out;             // optional branch output
  int br_rot;               // row pass: br_out takes element (i, j) at (i, (j - i) mod ncols), times (-1)^i
                            // (a column pass's alternating sums of it are the tile's diagonal sums)
  int br_d1;
  AwFactor fbr;
  int br_d2;
  AwFactor f2;
  int d2;
  AwFactor f3;
  double* red_line;         // column pass: per column, sum of Re
  double* red_cross;        // column pass: [block][row], sum of Re over the block's columns
  double* red_sq;           // column pass: [block], sum of Re(v*v)
  double2* col_alt;         // column pass: per column j, Sum_i (-1)^i v_ij (after f3)
  double2* alt_cross;       // column pass: [block][row i], Sum over the block's columns j of (-1)^j v_ij
  int lines_hint;           // column pass: columns per block (0: chosen for occupancy)
  int cluster;              // column pass: blocks per thread-block cluster; > 1 reduces alt_cross across the
                            // cluster through distributed shared memory ([cluster][row] partials)
  double2* diag_out;        // row pass: element (i, i) at the branch point
  double* red_abs2;         // row pass: [block], sum of |v|^2 at the branch point (or at the end)
  int abs2_end;             // take red_abs2 after f3 instead of at the branch point
  const int* stop;          // when non-zero the pass is skipped
  long long batch_elems;    // batched launches: elements per instance (blockIdx.y)
  long long batch_tab;      // ... table entries per instance
  int inst0;                // instance of blockIdx.y = 0 (a launch over a range of a batch's instances)
  int row_lines;            // row pass: rows per block (0: chosen from nrows)
  int tma;                  // column pass: stage the tile load and the store of `out` by TMA (tensor maps
                            // filled in by the launcher)
  int* err;                 // device error word: a bounded wait that ran out records its code here (or 0)
  int shape;                // 0: elements a thread (and so FFT radix) by the size rule; 1: the other choice
                            // (launchers return -9 where it does not exist)
  alignas(64) unsigned char tmap_in[128];   // CUtensorMap of `in`, then of `out` (launcher-written)
  alignas(64) unsigned char tmap_out[128];
} AwPassArgs;

// A grouped launch: the passes of up to AW_GROUP_MAX propagators of different line lengths (64 to
// AW_GROUP_LONGEST) run by one persistent kernel, each block walking work items (a member's tile of
// lines) in index order.  Every member computes with AW_GROUP_NT threads of 8 elements a tile of
// AW_GROUP_TILE elements (radix-8 stages).  Longer members fill the GPU with their own launches and are
// not grouped (aw_group_propagate runs their own step loop).
#define AW_GROUP_MAX 8
#define AW_GROUP_LONGEST 256
#define AW_GROUP_NT 128
#define AW_GROUP_TILE 1024
typedef struct AwGroupArgs {
  int count;
  int start[AW_GROUP_MAX + 1];  // first work item of each member; start[count]: the total
  int tiles_x[AW_GROUP_MAX];    // tiles along the member's lines (its work items are tiles_x x instances)
  AwPassArgs a[AW_GROUP_MAX];
} AwGroupArgs;

// Host-side launchers, one per precision (aw_pass_f64.cu / aw_pass_f32.cu).
// Returns 0 on success, or a negative code when the size is unsupported.
int aw_launch_row_pass_f64(const AwPassArgs* a, int batch, void* stream);
int aw_launch_col_pass_f64(const AwPassArgs* a, int batch, void* stream);
int aw_launch_row_pass_f32(const AwPassArgs* a, int batch, void* stream);
int aw_launch_col_pass_f32(const AwPassArgs* a, int batch, void* stream);
int aw_launch_row_pass_df(const AwPassArgs* a, int batch, void* stream);
int aw_launch_col_pass_df(const AwPassArgs* a, int batch, void* stream);
// grouped passes (row != 0: row passes): 0 on success, negative when a member's length is unsupported
int aw_launch_group_f64(const AwGroupArgs* g, int row, void* stream);
int aw_launch_group_f32(const AwGroupArgs* g, int row, void* stream);
int aw_launch_group_df(const AwGroupArgs* g, int row, void* stream);
// lines of one tile of a grouped pass for line length n (0: unsupported length)
int aw_group_tile_lines(int n);
// number of column blocks (rows of red_cross) the column pass uses for a given N (single instance)
int aw_col_pass_blocks(int nrows, int ncols, int f32);
// columns per column-pass block for `batch` instances
int aw_col_pass_lines(int nrows, int ncols, int batch, int f32);
// the most columns a column-pass block can hold (shared-memory limit)
// rows per row-pass block for a launch covering `rows_total` rows of length ncols (all instances)
int aw_row_pass_lines_for(int rows_total, int ncols, int f32);
int aw_col_pass_max_lines(int nrows, int ncols, int f32);
// number of rows one row-pass block holds for a row length ncols
int aw_row_pass_lines(int ncols, int f32);
// number of blocks of a row pass over nrows rows
int aw_row_pass_blocks(int nrows, int ncols, int f32);

#ifdef __cplusplus
}
#endif
