// FP64 step kernels, reference-exact variant: built with -fmad=false (see
// build.py), every operation rounded like the reference's host code.
#define DUGKS_EXACT 1
#include "fp64_step.cuh"
