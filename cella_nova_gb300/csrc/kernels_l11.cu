// Step kernels for grid side 2048.
#include "step_kernels.cuh"
CG_DEFINE_SIZE_OPS(11)
