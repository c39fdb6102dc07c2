// complex64 instantiations of the fused pass kernels
#include "aw_pass.cuh"

extern "C" int aw_launch_row_pass_f32(const AwPassArgs* a, int batch, void* stream) {
  return launch_row<float2>(a, batch, (cudaStream_t)stream);
}
extern "C" int aw_launch_col_pass_f32(const AwPassArgs* a, int batch, void* stream) {
  return launch_col<float2>(a, batch, (cudaStream_t)stream);
}
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
