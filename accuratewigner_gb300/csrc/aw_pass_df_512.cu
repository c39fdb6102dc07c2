// double-float pass kernels, line length 512
#include "aw_pass.cuh"

AW_SIZE_LAUNCHERS(dfc, df, 512)
