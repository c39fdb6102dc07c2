// double-float pass kernels, line length 4096
#include "aw_pass.cuh"

AW_SIZE_LAUNCHERS(dfc, df, 4096)
