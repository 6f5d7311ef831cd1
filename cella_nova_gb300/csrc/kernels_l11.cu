// Step kernels for grid side 2048.
#include "builder.cuh"
CG_DEFINE_SIZE_OPS(11)
