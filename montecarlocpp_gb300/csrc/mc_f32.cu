// FP32 flight kernels (FP64 tallies).
#define MC_REAL float
#include "mc_launch_impl.cuh"
