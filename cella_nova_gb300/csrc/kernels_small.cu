// Step kernels for grid sides 16 to 256 (test and small-creature sizes).
#include "builder.cuh"
CG_DEFINE_SIZE_OPS(4)
CG_DEFINE_SIZE_OPS(5)
CG_DEFINE_SIZE_OPS(6)
CG_DEFINE_SIZE_OPS(7)
CG_DEFINE_SIZE_OPS(8)
