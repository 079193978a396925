// Kernels of the RK2 step in the plain (FP64) form, and the precision-independent
// host helpers; see gt_kernels_impl.cuh.
#define GT_REAL double
#define GT_KERNELS_COMMON
#include "gt_kernels_impl.cuh"
