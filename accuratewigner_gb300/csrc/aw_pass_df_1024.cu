// double-float pass kernels, line length 1024
#include "aw_pass.cuh"

AW_SIZE_LAUNCHERS(dfc, df, 1024)
