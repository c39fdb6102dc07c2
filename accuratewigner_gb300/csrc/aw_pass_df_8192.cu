// double-float pass kernels, line length 8192
#include "aw_pass.cuh"

AW_SIZE_LAUNCHERS(dfc, df, 8192)
