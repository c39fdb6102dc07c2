// double-float pass kernels, line length 128
#include "aw_pass.cuh"

AW_SIZE_LAUNCHERS(dfc, df, 128)
