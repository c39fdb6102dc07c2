// complex128 state with double-float arithmetic: size dispatch of the fused pass kernels.
// The kernels themselves are instantiated in aw_pass_df_<sizes>.cu.
#include <cuda_runtime.h>

#include "aw_pass.h"

#define AW_DF_SIZES(M) M(32) M(64) M(128) M(256) M(512) M(1024) M(2048) M(4096) M(8192)
#define AW_DF_DECL(NN)                                                   \
  int aw_df_row_##NN(const AwPassArgs* a, int batch, cudaStream_t st); \
  int aw_df_col_##NN(const AwPassArgs* a, int batch, cudaStream_t st);
AW_DF_SIZES(AW_DF_DECL)

extern "C" int aw_launch_row_pass_df(const AwPassArgs* a, int batch, void* stream) {
  switch (a->ncols) {
#define AW_CASE(NN) \
  case NN: return aw_df_row_##NN(a, batch, (cudaStream_t)stream);
    AW_DF_SIZES(AW_CASE)
#undef AW_CASE
    default: return -1;
  }
}
extern "C" int aw_launch_col_pass_df(const AwPassArgs* a, int batch, void* stream) {
  switch (a->nrows) {
#define AW_CASE(NN) \
  case NN: return aw_df_col_##NN(a, batch, (cudaStream_t)stream);
    AW_DF_SIZES(AW_CASE)
#undef AW_CASE
    default: return -1;
  }
}
