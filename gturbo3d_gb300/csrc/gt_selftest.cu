// Self-test of the bounded device waits: the failure path a kernel takes when
// an mbarrier it waits on is never completed, exercised without a fault.
#include "gt_internal.h"
#include "gt_tma.cuh"

namespace gt {

// One thread waits on an mbarrier that nothing arrives at (no copy is
// issued), gives up after `limit` polls and records GT_ETIMEOUT in the error
// flag, as a kernel that stages its tiles with asynchronous copies does when
// they never land.  Nothing is in flight when it returns.
__global__ void k_wait_selftest(int* err, uint32_t limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    bool ok = false;
    for (uint32_t i = 0; i < limit && !ok; ++i) ok = mbar_try_wait(&bar, 0);
    if (!ok) raise_error(err, GT_ETIMEOUT);
    mbar_inval(&bar);
  }
}

int launch_wait_selftest(int* err, void* stream) {
  k_wait_selftest<<<1, 32, 0, (cudaStream_t)stream>>>(err, 1u << 12);
  return (int)cudaGetLastError();
}

}  // namespace gt
