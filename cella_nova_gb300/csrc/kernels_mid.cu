// Step kernels for grid sides 512 and 1024.
#include "builder.cuh"
CG_DEFINE_SIZE_OPS(9)
CG_DEFINE_SIZE_OPS(10)
