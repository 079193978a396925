// ALU issue-rate probe: the FP64 and FP32 ceilings of the transform passes.
//
// The plain (FP64) form of the step is bound by the FP64 pipe, not by HBM, so
// its roofline needs this GPU's FP64 add and fused multiply-add rates; they
// are measured here rather than taken from a datasheet.  Each thread runs
// eight independent dependency chains (enough to cover the pipe latency) over
// a grid of 8 blocks of 256 threads per SM; rates are warp-instruction counts
// times 32 lanes per second.
#include <cuda_runtime.h>

#include <cstdint>

#include "gt_internal.h"

namespace {

template <typename T, bool FMA>
__global__ void k_alu_chains(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x * (T)1e-7, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
  T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; ++i) {
    if (FMA) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    } else {
      x0 = x0 + b; x1 = x1 + a; x2 = x2 + b; x3 = x3 + a;
      x4 = x4 + b; x5 = x5 + a; x6 = x6 + b; x7 = x7 + a;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T, bool FMA>
int time_chains(int sms, double* rate) {
  const int grid = sms * 8, block = 256, iters = sizeof(T) == 8 ? 2000 : 40000;
  T* out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(T) * (size_t)grid * block);
  if (e != cudaSuccess) return (int)e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_alu_chains<T, FMA><<<grid, block>>>(out, 10, (T)0.999, (T)1e-3);   // warm-up
  cudaEventRecord(e0);
  k_alu_chains<T, FMA><<<grid, block>>>(out, iters, (T)0.999, (T)1e-3);
  cudaEventRecord(e1);
  e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return (int)e;
  *rate = (double)grid * block * iters * 8 / (ms * 1e-3) / 1e9;   // G thread-instructions/s
  return 0;
}

}  // namespace

extern "C" int gt_probe_alu(int32_t device, double* rates) {
  if (!rates) return GT_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return GT_ECUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return GT_ECUDA;
  if (time_chains<double, true>(sms, &rates[0]) || time_chains<double, false>(sms, &rates[1]) ||
      time_chains<float, true>(sms, &rates[2]) || time_chains<float, false>(sms, &rates[3]))
    return GT_ECUDA;
  return GT_OK;
}
