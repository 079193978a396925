// ALU issue-rate probe: the FP64 and FP32 ceilings of the transform passes.
//
// The plain (FP64) form of the step is bound by the FP64 pipe, not by HBM, so
// its roofline needs this GPU's FP64 add and fused multiply-add rates; they
// are measured here rather than taken from a datasheet.  Each thread runs
// eight independent dependency chains (enough to cover the pipe latency) over
// a grid of 8 blocks of 256 threads per SM; rates are warp-instruction counts
// times 32 lanes per second.
#include <cuda_runtime.h>

#include <algorithm>
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

// ===========================================================================
// Memory-pattern probe: copy kernels that move exactly the algorithmic bytes
// of each pass of the step, with the pass's tile shape and none of its
// arithmetic, timed per launch.  The DRAM rate of an access pattern depends on
// it (whole 128-byte rows of a contiguous line, 64- or 128-byte row segments of
// a column tile a plane apart), so each pass's rate is compared with the rate
// its own pattern allows on this GPU as well as with a plain copy.  Each
// thread moves 16-byte units (two FP32 or one FP64 complex value; a unit that
// straddles a limit moves element by element), loading a batch of rows (RB)
// before storing their results, so that several loads are in flight.
// ===========================================================================
#include "gt_handle.h"

namespace {

struct P9 {
  void* p[9];
};

template <typename C>
struct Unit {
  static constexpr int W = 16 / (int)sizeof(C);   // complex values per 16-byte unit
  C v[W];
};

// The W values at p[o] of columns X0.. with columns >= lim read as zero.
template <typename C>
__device__ __forceinline__ Unit<C> ld_unit(const C* __restrict__ p, size_t o, int X0, int lim) {
  Unit<C> u;
  constexpr int W = Unit<C>::W;
  if (X0 + W <= lim) {
    u = *reinterpret_cast<const Unit<C>*>(p + o);
  } else {
#pragma unroll
    for (int c = 0; c < W; ++c) u.v[c] = X0 + c < lim ? p[o + c] : C{0, 0};
  }
  return u;
}
template <typename C>
__device__ __forceinline__ void st_unit(C* __restrict__ p, size_t o, int X0, int lim, const Unit<C>& u) {
  constexpr int W = Unit<C>::W;
  if (X0 + W <= lim) {
    *reinterpret_cast<Unit<C>*>(p + o) = u;
  } else {
#pragma unroll
    for (int c = 0; c < W; ++c)
      if (X0 + c < lim) p[o + c] = u.v[c];
  }
}
template <typename C>
__device__ __forceinline__ Unit<C> scale(const Unit<C>& u, float s) {
  Unit<C> r;
#pragma unroll
  for (int c = 0; c < Unit<C>::W; ++c) r.v[c] = C{u.v[c].x * s, u.v[c].y * s};
  return r;
}

constexpr int kPatRows = 64;   // rows of a tile in flight per thread column

// z inverse pass: per tile (TX columns of row y), the three input fields at the
// kept rows (X < xcut[z][y]), the six outputs at every z for X < xcut[0][y].
template <typename C, int RB>
__global__ void k_pat_zinv(P9 f, gt::Geom g, const int32_t* __restrict__ xcut, const int32_t* __restrict__ tiles,
                           int TX) {
  constexpr int W = Unit<C>::W;
  const int TP = TX / W, xp = threadIdx.x % TP, t = threadIdx.x / TP;
  const int tile = tiles[2 * blockIdx.x], y = tiles[2 * blockIdx.x + 1];
  const int X0 = tile * TX + W * xp, ylim = xcut[y];
  if (X0 >= ylim) return;
  const size_t plane = (size_t)g.ny * g.nhp;
  for (int z0 = t; z0 < g.nz; z0 += RB * kPatRows) {
    Unit<C> a[RB][3];
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int z = z0 + b * kPatRows;
      const size_t o = (size_t)z * plane + (size_t)y * g.nhp + X0;
      const int lim = z < g.nz ? xcut[(size_t)z * g.ny + y] : 0;
#pragma unroll
      for (int q = 0; q < 3; ++q) a[b][q] = ld_unit(static_cast<const C*>(f.p[6 + q]), o, X0, lim);
    }
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int z = z0 + b * kPatRows;
      if (z >= g.nz) break;
      const size_t o = (size_t)z * plane + (size_t)y * g.nhp + X0;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        st_unit(static_cast<C*>(f.p[q]), o, X0, ylim, a[b][q]);
        st_unit(static_cast<C*>(f.p[3 + q]), o, X0, ylim, scale(a[b][q], 2.f));
      }
    }
  }
}

// y passes, in place per (x-tile, z-plane, field): inverse (dir = 1) reads the
// rows with X < xcut[0][y] and writes every row for X < xa; forward (dir = -1)
// reads every row for X < xa and writes the rows with X < xcut[0][y].
template <typename C, int RB>
__global__ void k_pat_y(P9 f, gt::Geom g, const int32_t* __restrict__ xcut, int xa, int TX, int dir) {
  constexpr int W = Unit<C>::W;
  const int TP = TX / W, xp = threadIdx.x % TP, t = threadIdx.x / TP;
  const int X0 = blockIdx.x * TX + W * xp;
  if (X0 >= xa) return;
  C* p = static_cast<C*>(f.p[blockIdx.z]);
  const size_t plane = (size_t)g.ny * g.nhp;
  for (int y0 = t; y0 < g.ny; y0 += RB * kPatRows) {
    Unit<C> u[RB];
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int y = y0 + b * kPatRows;
      const size_t o = (size_t)blockIdx.y * plane + (size_t)y * g.nhp + X0;
      const int cut = y < g.ny ? min(xa, xcut[y]) : 0;
      u[b] = ld_unit(p, o, X0, y < g.ny ? (dir > 0 ? cut : xa) : 0);
    }
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int y = y0 + b * kPatRows;
      if (y >= g.ny) break;
      const size_t o = (size_t)blockIdx.y * plane + (size_t)y * g.nhp + X0;
      const int cut = min(xa, xcut[y]);
      st_unit(p, o, X0, dir > 0 ? xa : cut, scale(u[b], 2.f));
    }
  }
}

// x pass: a group of 64 threads per pair of rows reads the six fields at
// kx < xa and writes three.
template <typename C>
__global__ void k_pat_x(P9 f, gt::Geom g, int xa) {
  constexpr int W = Unit<C>::W;
  const int grp = threadIdx.x >> 6, t = threadIdx.x & 63;
  const size_t pair = (size_t)blockIdx.x * (blockDim.x >> 6) + grp;
  if (2 * pair + 1 >= (size_t)g.ny * g.nz) return;
  for (int r = 0; r < 2; ++r) {
    const size_t ro = (2 * pair + r) * g.nhp;
    for (int X0 = W * t; X0 < xa; X0 += 64 * W) {
      Unit<C> u[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) u[q] = ld_unit(static_cast<const C*>(f.p[q]), ro + X0, X0, xa);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        Unit<C> s;
#pragma unroll
        for (int c = 0; c < W; ++c) s.v[c] = C{u[q].v[c].x + u[q + 3].v[c].y, u[q].v[c].y - u[q + 3].v[c].x};
        st_unit(static_cast<C*>(f.p[q]), ro + X0, X0, xa, s);
      }
    }
  }
}

// z forward pass: per tile, the three inputs at every z for X < xcut[0][y],
// the state read and the result written at the kept rows.
template <typename C, int RB>
__global__ void k_pat_zfwd(P9 f, gt::Geom g, const int32_t* __restrict__ xcut, const int32_t* __restrict__ tiles,
                           int TX) {
  constexpr int W = Unit<C>::W;
  const int TP = TX / W, xp = threadIdx.x % TP, t = threadIdx.x / TP;
  const int tile = tiles[2 * blockIdx.x], y = tiles[2 * blockIdx.x + 1];
  const int X0 = tile * TX + W * xp, ylim = xcut[y];
  if (X0 >= ylim) return;
  const size_t plane = (size_t)g.ny * g.nhp;
  for (int z0 = t; z0 < g.nz; z0 += RB * kPatRows) {
    Unit<C> s[RB][3];
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int z = z0 + b * kPatRows;
      const size_t o = (size_t)z * plane + (size_t)y * g.nhp + X0;
      const int lim = z < g.nz ? xcut[(size_t)z * g.ny + y] : 0;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const Unit<C> n = ld_unit(static_cast<const C*>(f.p[q]), o, X0, z < g.nz ? ylim : 0);
        const Unit<C> st = ld_unit(static_cast<const C*>(f.p[6 + q]), o, X0, lim);
#pragma unroll
        for (int c = 0; c < W; ++c) s[b][q].v[c] = C{n.v[c].x + st.v[c].x, n.v[c].y + st.v[c].y};
      }
    }
#pragma unroll
    for (int b = 0; b < RB; ++b) {
      const int z = z0 + b * kPatRows;
      if (z >= g.nz) break;
      const size_t o = (size_t)z * plane + (size_t)y * g.nhp + X0;
      const int lim = xcut[(size_t)z * g.ny + y];
#pragma unroll
      for (int q = 0; q < 3; ++q) st_unit(static_cast<C*>(f.p[6 + q]), o, X0, lim, s[b][q]);
    }
  }
}

template <typename C, typename L>
int time_pattern(cudaStream_t s, L launch, double* ms_out) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return GT_ECUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return GT_ECUDA;
  }
  launch();   // warm-up
  cudaEventRecord(e0, s);
  constexpr int reps = 3;
  for (int i = 0; i < reps; ++i) launch();
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return gtc::cuda_fail(e, "pattern probe");
  *ms_out = ms / reps;
  return GT_OK;
}

template <typename C, typename R>
int probe_patterns(gt_handle* h, const gt::DevTables<R>& tb, double* ms) {
  const gt::Geom& g = h->g;
  cudaStream_t s = h->stream;
  P9 f{};
  for (int i = 0; i < 6; ++i) f.p[i] = h->w[i];
  for (int i = 0; i < 3; ++i) f.p[6 + i] = h->c[i];
  const bool pruned = gtc::use_pruning(h);
  const int32_t* xcut = tb.xcut;
  const int xa = pruned ? tb.xa : g.nh;
  // the passes' tile widths: z tiles of 16 FP32 columns for z columns of 256
  // points or more (else 8), 4 FP64 columns; y tiles of 8 FP32 / 4 FP64 columns
  const int ztx = sizeof(C) == 8 ? (g.lnz >= 8 ? 16 : 8) : 4;
  const int ytx = sizeof(C) == 8 ? 8 : 4;
  int lg = 0;
  while ((1 << lg) < ztx) ++lg;
  const int zthreads = (ztx / Unit<C>::W) * kPatRows, ythreads = (ytx / Unit<C>::W) * kPatRows;
  // unpruned: every column of every row is active (the same kernels with a full-width tile list
  // would need one; the probe then reports the pruned-layout patterns only)
  if (!pruned) return GT_EINVAL;
  const unsigned ntiles = (unsigned)tb.nztl[lg];
  const int32_t* tiles = tb.ztl[lg];
  const unsigned ntxy = (unsigned)((xa + ytx - 1) / ytx);
  const unsigned xblocks = (unsigned)(((size_t)g.ny * g.nz / 2 + 3) / 4);
  // each pattern with one row per batch and with a batch of rows in flight; the faster counts
  int rc;
  double a = 0, b = 0;
  if ((rc = time_pattern<C>(s, [&] { k_pat_zinv<C, 1><<<ntiles, zthreads, 0, s>>>(f, g, xcut, tiles, ztx); }, &a)) ||
      (rc = time_pattern<C>(s, [&] { k_pat_zinv<C, 4><<<ntiles, zthreads, 0, s>>>(f, g, xcut, tiles, ztx); }, &b)))
    return rc;
  ms[0] = std::min(a, b);
  const dim3 gy6(ntxy, g.nz, 6), gy3(ntxy, g.nz, 3);
  if ((rc = time_pattern<C>(s, [&] { k_pat_y<C, 1><<<gy6, ythreads, 0, s>>>(f, g, xcut, xa, ytx, 1); }, &a)) ||
      (rc = time_pattern<C>(s, [&] { k_pat_y<C, 8><<<gy6, ythreads, 0, s>>>(f, g, xcut, xa, ytx, 1); }, &b)))
    return rc;
  ms[1] = std::min(a, b);
  if ((rc = time_pattern<C>(s, [&] { k_pat_x<C><<<xblocks, 256, 0, s>>>(f, g, xa); }, &ms[2]))) return rc;
  if ((rc = time_pattern<C>(s, [&] { k_pat_y<C, 1><<<gy3, ythreads, 0, s>>>(f, g, xcut, xa, ytx, -1); }, &a)) ||
      (rc = time_pattern<C>(s, [&] { k_pat_y<C, 8><<<gy3, ythreads, 0, s>>>(f, g, xcut, xa, ytx, -1); }, &b)))
    return rc;
  ms[3] = std::min(a, b);
  if ((rc = time_pattern<C>(s, [&] { k_pat_zfwd<C, 1><<<ntiles, zthreads, 0, s>>>(f, g, xcut, tiles, ztx); }, &a)) ||
      (rc = time_pattern<C>(s, [&] { k_pat_zfwd<C, 4><<<ntiles, zthreads, 0, s>>>(f, g, xcut, tiles, ztx); }, &b)))
    return rc;
  ms[4] = std::min(a, b);
  return GT_OK;
}

}  // namespace

extern "C" int gt_probe_patterns(gt_handle* h, double* ms) {
  if (!h || !ms) return GT_EINVAL;
  int rc = gtc::set_dev(h);
  if (rc) return rc;
  return h->mixed ? probe_patterns<float2>(h, h->t32, ms) : probe_patterns<double2>(h, h->t64, ms);
}
