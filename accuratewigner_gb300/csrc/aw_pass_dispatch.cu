// Size dispatch of the fused pass kernels, for the three arithmetic forms (complex128 on native FP64,
// complex128 in double-float, complex64).  The kernels of each (form, line length) are instantiated in
// their own translation unit, generated at build time from AW_SIZE_LAUNCHERS (aw_pass.cuh), so that
// the units compile in parallel.  The shape helpers below are host-only.
#include <cuda_runtime.h>

#include "aw_pass.cuh"

#define AW_DISPATCH_SIZES(M) M(32) M(64) M(128) M(256) M(512) M(1024) M(2048) M(4096) M(8192)
#define AW_DECL(TAG, NN)                                                    \
  int aw_##TAG##_row_##NN(const AwPassArgs* a, int batch, cudaStream_t st); \
  int aw_##TAG##_col_##NN(const AwPassArgs* a, int batch, cudaStream_t st);
#define AW_DECL_DF(NN) AW_DECL(df, NN)
#define AW_DECL_F64(NN) AW_DECL(f64, NN)
#define AW_DECL_F32(NN) AW_DECL(f32, NN)
AW_DISPATCH_SIZES(AW_DECL_DF)
AW_DISPATCH_SIZES(AW_DECL_F64)
AW_DISPATCH_SIZES(AW_DECL_F32)

#define AW_LAUNCHERS(TAG)                                                              \
  extern "C" int aw_launch_row_pass_##TAG(const AwPassArgs* a, int batch, void* stream) { \
    switch (a->ncols) {                                                                \
      AW_DISPATCH_SIZES(AW_ROW_CASE_##TAG)                                             \
      default: return -1;                                                              \
    }                                                                                  \
  }                                                                                    \
  extern "C" int aw_launch_col_pass_##TAG(const AwPassArgs* a, int batch, void* stream) { \
    switch (a->nrows) {                                                                \
      AW_DISPATCH_SIZES(AW_COL_CASE_##TAG)                                             \
      default: return -1;                                                              \
    }                                                                                  \
  }
#define AW_ROW_CASE_df(NN) \
  case NN: return aw_df_row_##NN(a, batch, (cudaStream_t)stream);
#define AW_COL_CASE_df(NN) \
  case NN: return aw_df_col_##NN(a, batch, (cudaStream_t)stream);
#define AW_ROW_CASE_f64(NN) \
  case NN: return aw_f64_row_##NN(a, batch, (cudaStream_t)stream);
#define AW_COL_CASE_f64(NN) \
  case NN: return aw_f64_col_##NN(a, batch, (cudaStream_t)stream);
#define AW_ROW_CASE_f32(NN) \
  case NN: return aw_f32_row_##NN(a, batch, (cudaStream_t)stream);
#define AW_COL_CASE_f32(NN) \
  case NN: return aw_f32_col_##NN(a, batch, (cudaStream_t)stream);
AW_LAUNCHERS(df)
AW_LAUNCHERS(f64)
AW_LAUNCHERS(f32)

extern "C" int aw_col_pass_lines(int nrows, int ncols, int batch, int f32) {
  return choose_col_lines(nrows, ncols, batch, f32 ? 8 : 16);
}
extern "C" int aw_col_pass_blocks(int nrows, int ncols, int f32) {
  return ncols / aw_col_pass_lines(nrows, ncols, 1, f32);
}
extern "C" int aw_row_pass_lines(int ncols, int f32) { return choose_row_lines(ncols, f32 ? 8 : 16); }
extern "C" int aw_row_pass_lines_for(int rows_total, int ncols, int f32) {
  return choose_row_lines(rows_total, ncols, f32 ? 8 : 16);
}
extern "C" int aw_row_pass_blocks(int nrows, int ncols, int f32) {
  const int l = choose_row_lines(nrows, ncols, f32 ? 8 : 16);
  return l > 0 ? nrows / l : -1;
}
extern "C" int aw_col_pass_max_lines(int nrows, int ncols, int f32) { return max_col_lines(nrows, ncols, f32 ? 8 : 16); }
// lines of a grouped pass's tile (aw_group.cuh: 2048 elements)
extern "C" int aw_group_tile_lines(int n) {
  return (n >= 64 && n <= AW_GROUP_LONGEST && !(n & (n - 1))) ? AW_GROUP_TILE / n : 0;
}
