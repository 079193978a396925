// gt_energy_noalloc: the kinetic-energy reduction of gt_energy for callers
// that cannot allocate device memory.
//
// Who needs it: a Fortran driver whose device arrays are owned by another
// runtime (an OpenACC data region, a pooled allocator that has reserved the
// HBM) holds the spectral fields on the device but may not create a handle,
// whose constructor allocates, and must not call cudaMalloc/cudaFree inside
// its time loop, where they would synchronise the device or fail under the
// other runtime's reservation.  This entry point takes the caller's device
// arrays and stream and allocates nothing: its scratch is the file-scope
// array below, reserved when the library is loaded and held by every GPU
// that loads the library until the process exits.
//
// The scratch holds one partial sum per (y, z) row, so it bounds the grid:
// at most kNoAllocMaxRows = 262144 rows (e.g. NY = NZ = 512), 6 MiB.  Every
// slot a call reads is written earlier in the same call, so nothing needs
// clearing between calls.  All calls on a device share the one array: calls
// that overlap on the GPU (different streams, or different host threads
// without ordering) race on it and must be serialised by the caller.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include <cuda.h>

#include "gt_internal.h"

namespace {

constexpr long long kNoAllocMaxRows = 262144;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxRows * 3];

// Host-side device addresses of g_noalloc_scratch, one per device, each
// tagged with the id of the CUDA context it was looked up in.  The symbol's
// name in host code is only a stand-in; the address must come from
// cudaGetSymbolAddress with the device current.  A new primary context (after
// cudaDeviceReset, or after the context was released and created again)
// reloads the module and may place the array elsewhere, so a lookup is reused
// only while the current context's id matches its tag.
struct ScratchSlot {
  double* addr = nullptr;
  unsigned long long ctx_id = 0;
};
ScratchSlot g_scratch_slot[kMaxDevices];
std::mutex g_scratch_mu;

using PFN_ctxGetCurrent = CUresult (*)(CUcontext*);
using PFN_ctxGetId = CUresult (*)(CUcontext, unsigned long long*);

// Id of the calling thread's current context (driver entry points looked up
// through the runtime, so the library need not link libcuda); false when it
// cannot be read, in which case the address is looked up on every call.
bool current_ctx_id(unsigned long long* id) {
  static PFN_ctxGetCurrent get_current = nullptr;
  static PFN_ctxGetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_ctxGetCurrent>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_ctxGetId>(p);
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

void fail_msg(const char* msg) { gt::set_last_error(msg); }

int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GT_ECUDA;
  if (dev < 0 || dev >= kMaxDevices) return GT_EINVAL;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long id = 0;
  const bool have_id = current_ctx_id(&id);
  ScratchSlot& slot = g_scratch_slot[dev];
  if (!slot.addr || !have_id || slot.ctx_id != id) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      char m[160];
      std::snprintf(m, sizeof m, "gt_energy_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
      fail_msg(m);
      return GT_ECUDA;
    }
    slot.addr = static_cast<double*>(p);
    slot.ctx_id = have_id ? id : 0;
  }
  *out = slot.addr;
  return GT_OK;
}

// One warp per (y, z) row: E_c of the row's modes, summed over the lanes by a
// fixed shuffle tree, written to the row's slot.
__global__ void k_energy_rows(const double2* __restrict__ b0, const double2* __restrict__ b1,
                              const double2* __restrict__ b2, int nx, int ny, int nz, double dkx,
                              double dky, double dkz, double* __restrict__ rows_out) {
  const int nh = nx / 2 + 1;
  const long long nrows = (long long)ny * nz;
  const int lane = threadIdx.x & 31;
  const long long row = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= nrows) return;
  const int y = (int)(row % ny), z = (int)(row / ny);
  const double ky = (y <= ny / 2 ? (double)y : (double)(y - ny)) * dky;
  const double kz = (z <= nz / 2 ? (double)z : (double)(z - nz)) * dkz;
  double e0 = 0.0, e1 = 0.0, e2 = 0.0;
  for (int X = lane; X < nh; X += 32) {
    const long long o = row * nh + X;
    const double2 a = b0[o], b = b1[o], c = b2[o];
    const double kx = (double)X * dkx;
    const double ux0 = -ky * c.y + kz * b.y, uy0 = ky * c.x - kz * b.x;
    const double ux1 = -kz * a.y + kx * c.y, uy1 = kz * a.x - kx * c.x;
    const double ux2 = -kx * b.y + ky * a.y, uy2 = kx * b.x - ky * a.x;
    const double fac = (X == 0 || X == nh - 1) ? 0.5 : 1.0;
    e0 += fac * (ux0 * ux0 + uy0 * uy0);
    e1 += fac * (ux1 * ux1 + uy1 * uy1);
    e2 += fac * (ux2 * ux2 + uy2 * uy2);
  }
  for (int off = 16; off > 0; off >>= 1) {
    e0 += __shfl_down_sync(0xffffffffu, e0, off);
    e1 += __shfl_down_sync(0xffffffffu, e1, off);
    e2 += __shfl_down_sync(0xffffffffu, e2, off);
  }
  if (lane == 0) {
    rows_out[3 * row] = e0;
    rows_out[3 * row + 1] = e1;
    rows_out[3 * row + 2] = e2;
  }
}

// One block: thread t sums rows t, t + 256, ... in order, then a fixed tree.
__global__ void k_energy_rows_sum(const double* __restrict__ rows_in, long long nrows,
                                  double* __restrict__ out) {
  __shared__ double red[3][256];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (long long r = threadIdx.x; r < nrows; r += blockDim.x) {
    s0 += rows_in[3 * r];
    s1 += rows_in[3 * r + 1];
    s2 += rows_in[3 * r + 2];
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  red[2][threadIdx.x] = s2;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if ((int)threadIdx.x < st)
      for (int c = 0; c < 3; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 3) out[threadIdx.x] = red[threadIdx.x][0];
}

bool pow2_in_range(int n) { return n >= 8 && n <= 1024 && (n & (n - 1)) == 0; }

}  // namespace

extern "C" {

int gt_energy_noalloc(const double* bx, const double* by, const double* bz, int32_t nx,
                      int32_t ny, int32_t nz, double xlx, double xly, double xlz,
                      double* energy_out, void* stream) {
  if (!bx || !by || !bz || !energy_out) {
    fail_msg("gt_energy_noalloc: null pointer");
    return GT_EINVAL;
  }
  if (!pow2_in_range(nx) || !pow2_in_range(ny) || !pow2_in_range(nz) || !(xlx > 0) ||
      !(xly > 0) || !(xlz > 0)) {
    fail_msg("gt_energy_noalloc: grid sides must be powers of two in [8, 1024] and box lengths positive");
    return GT_EINVAL;
  }
  const long long nrows = (long long)ny * nz;
  if (nrows > kNoAllocMaxRows) {
    char m[160];
    std::snprintf(m, sizeof m, "gt_energy_noalloc: NY*NZ = %lld rows exceeds the fixed scratch of %lld rows",
                  nrows, kNoAllocMaxRows);
    fail_msg(m);
    return GT_EINVAL;
  }
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  const double two_pi = 2.0 * gt::kPiRef;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int threads = 256;
  const long long blocks = (nrows + 7) / 8;
  k_energy_rows<<<(unsigned)blocks, threads, 0, s>>>(reinterpret_cast<const double2*>(bx),
                                                       reinterpret_cast<const double2*>(by),
                                                       reinterpret_cast<const double2*>(bz), nx,
                                                       ny, nz, two_pi / xlx, two_pi / xly,
                                                       two_pi / xlz, scratch);
  k_energy_rows_sum<<<1, 256, 0, s>>>(scratch, nrows, energy_out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    char m[160];
    std::snprintf(m, sizeof m, "gt_energy_noalloc: %s", cudaGetErrorString(e));
    fail_msg(m);
    return GT_ECUDA;
  }
  return GT_OK;
}

}  // extern "C"
