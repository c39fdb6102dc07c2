// complex128 instantiations of the fused pass kernels
#include "aw_pass.cuh"

extern "C" int aw_launch_row_pass_f64(const AwPassArgs* a, int batch, void* stream) {
  return launch_row<double2>(a, batch, (cudaStream_t)stream);
}
extern "C" int aw_launch_col_pass_f64(const AwPassArgs* a, int batch, void* stream) {
  return launch_col<double2>(a, batch, (cudaStream_t)stream);
}
