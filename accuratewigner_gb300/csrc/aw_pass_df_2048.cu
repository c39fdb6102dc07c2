// double-float pass kernels, line length 2048
#include "aw_pass.cuh"

AW_SIZE_LAUNCHERS(dfc, df, 2048)
