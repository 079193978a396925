// Kernels of the RK2 step in the mixed (FP32) form; see gt_kernels_impl.cuh.
#define GT_REAL float
#include "gt_kernels_impl.cuh"
