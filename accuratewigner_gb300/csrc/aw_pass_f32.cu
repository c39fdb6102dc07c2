// complex64 instantiations of the fused pass kernels
#include "aw_pass.cuh"

extern "C" int aw_launch_row_pass_f32(const AwPassArgs* a, int batch, void* stream) {
  return launch_row<float2>(a, batch, (cudaStream_t)stream);
}
extern "C" int aw_launch_col_pass_f32(const AwPassArgs* a, int batch, void* stream) {
  return launch_col<float2>(a, batch, (cudaStream_t)stream);
}
extern "C" int aw_col_pass_blocks(int nrows, int ncols, int f32) {
  return f32 ? col_blocks<float2>(nrows, ncols) : col_blocks<double2>(nrows, ncols);
}
extern "C" int aw_row_pass_lines(int ncols, int f32) {
  return f32 ? row_lines<float2>(ncols) : row_lines<double2>(ncols);
}
extern "C" int aw_row_pass_blocks(int nrows, int ncols, int f32) {
  const int l = aw_row_pass_lines(ncols, f32);
  return l > 0 ? nrows / l : -1;
}
