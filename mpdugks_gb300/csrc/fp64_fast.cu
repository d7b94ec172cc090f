// FP64 step kernels, fast variant: FMA contraction and reciprocal multiplies.
#define DUGKS_EXACT 0
#include "fp64_step.cuh"
