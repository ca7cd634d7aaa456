// FP64 flight kernels; built with --fmad=false so that products and sums
// round like the CPU oracle's.
#define MC_REAL double
#include "mc_launch_impl.cuh"
