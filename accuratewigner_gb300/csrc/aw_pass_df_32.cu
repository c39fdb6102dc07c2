// double-float pass kernels, line length 32
#include "aw_pass.cuh"

AW_SIZE_LAUNCHERS(dfc, df, 32)
