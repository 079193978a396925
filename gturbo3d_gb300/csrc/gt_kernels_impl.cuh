// Kernels of the RK2 integrating-factor step and their launchers.
//
// One nonlinear-term evaluation nlt(a; bcor) (nlt.f90:16-89) is five passes
// over HBM, each a batch of 1D FFT lines with the pointwise work fused at
// the pass boundaries:
//
//   1. k_zinv_curl  : per (x-tile, y) column block, u = i k x a and w = k^2 a
//                     formed on load (produ.f90:44-63, nlt.f90:26-40), then
//                     the inverse z transform of all six fields.
//   2. k_spass2     : inverse y transform of the six fields, in place (FP32,
//                     two columns per thread; k_spass for FP64).
//   3. k_xbatch     : per pair of (y,z) rows, the six C2R x transforms (two
//                     fields per complex FFT, a row's three packed lines as
//                     one three-line transform), u x w in registers
//                     (produ.f90:9-28), the three R2C x transforms and the
//                     1/(NX NY NZ) scaling (fft_dir.f90:17-25); real space
//                     never reaches HBM (k_xfused: the lines one by one;
//                     k_xcross: three thread groups per row pair).
//   4. k_spass2     : forward y transform of the three fields.
//   5. k_zfwd_epi   : forward z transform, then per mode the Coriolis term
//                     (nlt.f90:67-81), invcurl (produ.f90:79-101), trunc
//                     (trunc.f90:10-28) and, in a time step, the
//                     integrating-factor update step1 (rkstep.f90:30-48) or
//                     step2 (rkstep.f90:86-104), written straight into the
//                     stage or state buffers.
//
// With the 2/3 truncation the passes visit only the modes that can be
// nonzero (tile lists for the z passes, kx < xa for the y and x passes).
// Spectral fields are [nz][ny][nhp] complex, x fastest, rows padded to a
// multiple of 128 bytes; columns nh..nhp-1 are never read or written.
#include <cooperative_groups.h>
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <type_traits>

#include "gt_fft.cuh"
#include "gt_internal.h"
#include "gt_tma.cuh"

namespace gt {

struct Ptr6 {
  void* p[6];
  // Element i by selects: a run-time index into the parameter array would
  // make the compiler copy the array to local memory.
  __device__ __forceinline__ void* at(int i) const {
    void* r = p[0];
#pragma unroll
    for (int k = 1; k < 6; ++k)
      if (i == k) r = p[k];
    return r;
  }
};

// Element offset of member m's fields in a batched launch (0 for one member).
__device__ __forceinline__ size_t member_offset(long long mstride, unsigned m) {
  return mstride ? (size_t)m * (size_t)mstride : 0;
}

// A batched launch's member m: its own integrating factor and scalars.
template <typename R>
__device__ __forceinline__ void member_tables(const Batch<R>& bt, unsigned m, DevTables<R>& tb) {
  if (!bt.nmem) return;
  tb.emk = bt.emk + (size_t)m * bt.emk_len;
  tb.omega = bt.scal[3 * m];
  tb.dt = bt.scal[3 * m + 1];
  tb.dt2 = bt.scal[3 * m + 2];
}

constexpr int kSmemBudget = 200 * 1024;
// An explicitly requested tile width may use the whole per-block opt-in (227
// KB on GB300), e.g. 16-column z tiles of three 512-row fields (216 KB, one
// block per SM, 128-byte row segments).
constexpr int kSmemForced = 227 * 1024;

template <typename R> constexpr int max_threads() { return sizeof(R) == 8 ? 512 : 1024; }
// Block size bound of the strided single-region passes (y passes, w = k^2 a).
constexpr int kSpassThreads = 256;
// x passes: at most 3 x (N/8) x P threads with P row pairs chosen so that the
// block stays within 256 threads (192 for N <= 512, 384 for N = 1024); the
// register budget per thread is about 80 (FP32) or 168 (FP64).
template <int LG> constexpr int xcross_threads() { return LG >= 10 ? 384 : 192; }
template <typename R, int LG> constexpr int xcross_min_blocks() {
  return 65536 / (xcross_threads<LG>() * (sizeof(R) == 8 ? 168 : 80)) > 0
             ? 65536 / (xcross_threads<LG>() * (sizeof(R) == 8 ? 168 : 80))
             : 1;
}

static int ilog2i(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

// ---------------------------------------------------------------------------
// Pass 1: u = curl a, w = k^2 a, inverse z transform of the six fields.
// Block: (L/8) x TX threads; thread (t, x) owns positions z = t + i L/8 of
// column X = tile*TX + x.  Shared memory: three [nz][TX] regions.
// ---------------------------------------------------------------------------
// W columns per thread (1, or 2 for FP32: 16-byte accesses, twiddles and
// index arithmetic shared); E holds one position of those columns.
template <typename R, int W> struct ColVec { using type = Cplx<R>; };
template <typename R> struct ColVec<R, 2> { using type = CPair<R>; };
template <typename R, int W> using ColT = typename ColVec<R, W>::type;

__device__ __forceinline__ float2& col(float2& e, int) { return e; }
__device__ __forceinline__ double2& col(double2& e, int) { return e; }
template <typename R> __device__ __forceinline__ Cplx<R>& col(CPair<R>& e, int c) { return c ? e.b : e.a; }

// The W columns X0.. of one position at p[o]; columns >= lim read as zero.
template <typename R, int W>
__device__ __forceinline__ ColT<R, W> load_cols(const Cplx<R>* __restrict__ p, size_t o, int X0, int lim) {
  using C = Cplx<R>;
  if constexpr (W == 1) {
    return X0 < lim ? p[o] : C{0, 0};
  } else {
    if (X0 + 1 < lim) return *reinterpret_cast<const CPair<R>*>(p + o);
    return CPair<R>{X0 < lim ? p[o] : C{0, 0}, C{0, 0}};
  }
}
// Stores the columns < lim of one position.
template <typename R, int W>
__device__ __forceinline__ void store_cols(Cplx<R>* __restrict__ p, size_t o, int X0, int lim, const ColT<R, W>& v) {
  if constexpr (W == 1) {
    if (X0 < lim) p[o] = v;
  } else {
    if (X0 + 1 < lim) {
      *reinterpret_cast<CPair<R>*>(p + o) = v;
    } else if (X0 < lim) {
      p[o] = v.a;
    }
  }
}

// The same columns copied asynchronously into a shared-memory slot: the
// slot receives what load_cols returns (columns >= lim zero-filled).
template <typename R, int W>
__device__ __forceinline__ void load_cols_async(ColT<R, W>* sdst, const Cplx<R>* __restrict__ p, size_t o,
                                                int X0, int lim) {
  constexpr int B = (int)sizeof(ColT<R, W>);
  constexpr int CB = (int)sizeof(Cplx<R>);
  const int n = X0 + W <= lim ? B : (X0 < lim ? (lim - X0) * CB : 0);
  cp_async<B>(sdst, p + o, n);
}

// Columns per thread of the z inverse pass: 2 for FP32, 1 for FP64.  The z
// forward pass keeps one column per thread: its epilogue works column by
// column, and pairs measured slower there (0.49 ms against 0.46 ms at 512^3).
template <typename R> constexpr int zcols() { return sizeof(R) == 4 ? 2 : 1; }
template <typename R> constexpr int zfwd_cols() { return 1; }

template <typename R, int LGZ>
__global__ void __launch_bounds__(max_threads<R>() / zcols<R>())
k_zinv_curl(Ptr6 a, Ptr6 w, DevTables<R> tb, Geom g, int lgTX, int pruned, const int32_t* __restrict__ tiles,
            int k2part, long long mstride) {
  using C = Cplx<R>;
  constexpr int W = zcols<R>();
  using E = ColT<R, W>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  int tile = blockIdx.x, y = blockIdx.y;
  if (pruned) {
    tile = tiles[2 * blockIdx.x];
    y = tiles[2 * blockIdx.x + 1];
  }
  const int X0 = tile * TX + W * xp;
  const int ylim = pruned ? tb.xcut[y] : g.nh;   // columns with data in this y row
  const bool valid = X0 < ylim;
  constexpr int T = 1 << (LGZ - 3);
  const size_t plane = (size_t)g.ny * g.nhp;
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0) + member_offset(mstride, pruned ? blockIdx.y : blockIdx.z);
  const int reg = strided_rows(1 << LGZ) * TP;
  E* S0 = sm;
  E* S1 = sm + reg;
  E* S2 = sm + 2 * reg;
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  const C* a0 = reinterpret_cast<const C*>(a.p[0]);
  const C* a1 = reinterpret_cast<const C*>(a.p[1]);
  const C* a2 = reinterpret_cast<const C*>(a.p[2]);
  R kx[W], kxs[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    const bool in = X0 + c < ylim;
    kx[c] = in ? tb.fkx[X0 + c] : (R)0;
    kxs[c] = in ? tb.fkxs[X0 + c] : (R)0;
  }
  const R ky = tb.fky[y], kys = tb.fkys[y];
  E v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int z = t + i * T;
    const int lim = valid ? (pruned ? tb.xcut[(size_t)z * g.ny + y] : g.nh) : 0;
    const size_t o = (size_t)z * plane + base;
    E ax = load_cols<R, W>(a0, o, X0, lim), ay = load_cols<R, W>(a1, o, X0, lim),
      az = load_cols<R, W>(a2, o, X0, lim);
    const R kz = tb.fkz[z];
    E ux, uy, uz;
#pragma unroll
    for (int c = 0; c < W; ++c) {
      const C px = col(ax, c), py = col(ay, c), pz = col(az, c);
      col(ux, c) = C{-ky * pz.y + kz * py.y, ky * pz.x - kz * py.x};
      col(uy, c) = C{-kz * px.y + kx[c] * pz.y, kz * px.x - kx[c] * pz.x};
      col(uz, c) = C{-kx[c] * py.y + ky * px.y, kx[c] * py.x - ky * px.x};
    }
    v[i] = ux;
    S1[idx(z)] = uy;
    S2[idx(z)] = uz;
  }
  // The k^2 part re-reads a_c; its columns are copied asynchronously into
  // region c as soon as the u_c transform has finished with that region (its
  // last reads precede the transform's final barrier), so the copies run
  // behind the remaining u transforms instead of stalling the k^2 ones.
  auto prefetch = [&](int c3, E* S) {
    const C* ac = reinterpret_cast<const C*>(a.at(c3));
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int z = t + i * T;
      const int lim = valid ? (pruned ? tb.xcut[(size_t)z * g.ny + y] : g.nh) : 0;
      load_cols_async<R, W>(S + idx(z), ac, (size_t)z * plane + base, X0, lim);
    }
    cp_async_commit();
  };
  C* out0 = reinterpret_cast<C*>(w.p[0]);
  fft_line_ct<+1, R, LGZ>(v, t, tw, S0, idx);
#pragma unroll
  for (int i = 0; i < 8; ++i) store_cols<R, W>(out0, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
  if (k2part) prefetch(0, S0);   // behind this field's stores in the load/store queue
  for (int f = 1; f < 3; ++f) {
    E* S = f == 1 ? S1 : S2;
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
    __syncthreads();
    fft_line_ct<+1, R, LGZ>(v, t, tw, S, idx);
    C* out = reinterpret_cast<C*>(w.at(f));
#pragma unroll
    for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
    if (k2part) prefetch(f, S);
  }
  if (!k2part) return;   // w = k^2 a by k_zk2 (no barrier follows)
  for (int c3 = 0; c3 < 3; ++c3) {
    E* S = c3 == 0 ? S0 : (c3 == 1 ? S1 : S2);
    cp_async_wait(2 - c3);   // this thread's copies of a_c3 have landed
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int z = t + i * T;
      E av = S[idx(z)];
      const R kzs = tb.fkzs[z];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        const R k2 = (kxs[c] + kys) + kzs;
        const C q = col(av, c);
        col(av, c) = C{k2 * q.x, k2 * q.y};
      }
      v[i] = av;
    }
    __syncthreads();   // every thread holds its inputs before the exchanges overwrite the region
    fft_line_ct<+1, R, LGZ>(v, t, tw, S, idx);
    C* out = reinterpret_cast<C*>(w.at(3 + c3));
#pragma unroll
    for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
  }
}

// ---------------------------------------------------------------------------
// Pass 1 with TMA-loaded inputs (FP32, pruned, 16-column tiles, z_tma bit 2).
// The tile's kept z-rows of a_0..a_2 (z <= zc and z >= nz - zc, zc from the
// tile list) arrive by tensor copies of 32-row boxes issued by one thread,
// an mbarrier per field, into dense regions (16 FP32 columns make whole
// 128-byte rows); for the k^2 part each a_c is copied again, by TMA, into the
// region the u_c transform has finished with.  Rows a box does not cover are
// never read: every read of an input row is masked by the row's kept prefix,
// as the cp.async copies of k_zinv_curl zero-fill them.  Bounded waits.
// ---------------------------------------------------------------------------
// Dense shared tile of a TMA-loaded z pass: element e of column x of a
// [rows][2^lg] tile (rows of 16 FP32 columns are whole 128-byte lines, so the
// transforms' warp accesses cover whole rows and need no padding rows).
struct DenseIdxLg {
  int lg, x;
  __device__ __forceinline__ int operator()(int e) const { return (e << lg) + x; }
};
constexpr int kZTmaLgTX = 4;   // 16 columns per tile
constexpr int kZBoxRows = 32;

// Tensor maps of pass 1's six outputs, for its tensor stores.
struct ZOutMaps {
  CUtensorMap m[6];
};

// TST: the six outputs leave by tensor stores from the tile's regions (z_tma
// bit 4) instead of per-thread stores.  A transformed field is written into
// its region and one thread issues the stores; the threads go on with the next
// transform while the stores drain, and a_c is copied again into region c for
// the k^2 part once region c's store has read it.  The stores write whole
// 16-column boxes: the tile's columns at or beyond the row's limit receive the
// zeros their transforms produce, which no later pass reads (the y pass masks
// its inputs by the same limits).
template <int LGZ, bool TST = false>
__global__ void __launch_bounds__(1 << LGZ > 1024 ? 1024 : (1 << LGZ), 1)
k_zinv_tma(const __grid_constant__ CUtensorMap m0, const __grid_constant__ CUtensorMap m1,
           const __grid_constant__ CUtensorMap m2, const __grid_constant__ ZOutMaps om, Ptr6 w,
           DevTables<float> tb, Geom g, const int32_t* __restrict__ tiles, const int32_t* __restrict__ tzc,
           int* err) {
  using R = float;
  using C = float2;
  constexpr int W = 2;
  using E = CPair<float>;
  constexpr int L = 1 << LGZ, T = L / 8;
  constexpr int TX = 1 << kZTmaLgTX, lgTP = kZTmaLgTX - 1, TP = TX / 2;
  extern __shared__ __align__(128) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + (size_t)3 * L * TP * sizeof(E));
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  const int tile = tiles[2 * blockIdx.x], y = tiles[2 * blockIdx.x + 1];
  const int zc = tzc[blockIdx.x];
  // boxes: rows [0, hend) and [tstart, L), whole boxes, no overlap
  const int hend = min(L, (zc / kZBoxRows + 1) * kZBoxRows);
  const int tstart = max(hend, (L - zc) / kZBoxRows * kZBoxRows);
  const int nbox = hend / kZBoxRows + (L - tstart) / kZBoxRows;
  const int X0 = tile * TX + W * xp;
  const int ylim = tb.xcut[y];
  const bool valid = X0 < ylim;
  const size_t plane = (size_t)g.ny * g.nhp;
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0);
  const int reg = L * TP;
  const DenseIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  const CUtensorMap* m[3] = {&m0, &m1, &m2};
  // thread 0: the kept rows of field c into region c, completing bar[k]
  auto load_field = [&](int c, int k) {
    mbar_arrive_expect_tx(&bar[k], (uint32_t)(nbox * kZBoxRows * TX * sizeof(C)));
    for (int z0 = 0; z0 < hend; z0 += kZBoxRows)
      tma_load_3d(sm + c * reg + z0 * TP, m[c], tile * 2 * TX, y, z0, &bar[k]);
    for (int z0 = tstart; z0 < L; z0 += kZBoxRows)
      tma_load_3d(sm + c * reg + z0 * TP, m[c], tile * 2 * TX, y, z0, &bar[k]);
  };
  auto wait = [&](int k) {
    if (!mbar_wait(&bar[k], 0)) {   // bounded: record it, and give the copies one more bounded wait
      raise_error(err, GT_ETIMEOUT);
      mbar_wait(&bar[k], 0);
    }
  };
  if (threadIdx.x == 0) {
    for (int k = 0; k < 6; ++k) mbar_init(&bar[k], 1);
    fence_mbar_init();
    for (int c = 0; c < 3; ++c) load_field(c, c);
  }
  __syncthreads();   // the barriers are initialised before anyone waits on them
  R kx[W], kxs[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    const bool in = X0 + c < ylim;
    kx[c] = in ? tb.fkx[X0 + c] : (R)0;
    kxs[c] = in ? tb.fkxs[X0 + c] : (R)0;
  }
  const R ky = tb.fky[y], kys = tb.fkys[y];
  // the value of column pair X0 at row z of region c, zero outside the row's kept prefix
  auto kept = [&](const E* S, int z, int lim) {
    E u = S[idx(z)];
    if (X0 + 1 >= lim) {
      u.b = C{0, 0};
      if (X0 >= lim) u.a = C{0, 0};
    }
    return u;
  };
  wait(0);
  wait(1);
  wait(2);
  E* S0 = sm;
  E* S1 = sm + reg;
  E* S2 = sm + 2 * reg;
  E v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int z = t + i * T;
    const int lim = valid ? tb.xcut[(size_t)z * g.ny + y] : 0;
    E ax = kept(S0, z, lim), ay = kept(S1, z, lim), az = kept(S2, z, lim);
    const R kz = tb.fkz[z];
    E ux, uy, uz;
#pragma unroll
    for (int c = 0; c < W; ++c) {
      const C px = col(ax, c), py = col(ay, c), pz = col(az, c);
      col(ux, c) = C{-ky * pz.y + kz * py.y, ky * pz.x - kz * py.x};
      col(uy, c) = C{-kz * px.y + kx[c] * pz.y, kz * px.x - kx[c] * pz.x};
      col(uz, c) = C{-kx[c] * py.y + ky * px.y, kx[c] * py.x - ky * px.x};
    }
    v[i] = ux;
    S1[idx(z)] = uy;   // this thread's own slots, read just above
    S2[idx(z)] = uz;
  }
  __syncthreads();   // every thread has read region 0 before the exchanges overwrite it
  constexpr int OB = L < 256 ? L : 256;   // rows per store box
  // thread 0: region S, all L rows, to output k by tensor stores, one bulk group
  auto store_field = [&](const E* S, int k) {
    for (int z0 = 0; z0 < L; z0 += OB) tma_store_3d(&om.m[k], S + z0 * TP, tile * 2 * TX, y, z0);
    bulk_commit();
  };
  // every thread: its transformed column pair into region S (the transform's
  // last exchange read is behind a barrier), ordered before the tensor stores
  auto put = [&](E* S) {
#pragma unroll
    for (int i = 0; i < 8; ++i) S[idx(t + i * T)] = v[i];
    fence_proxy_async_smem();
    __syncthreads();
  };
  for (int f = 0; f < 3; ++f) {
    E* S = f == 0 ? S0 : (f == 1 ? S1 : S2);
    if (f > 0) {
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
      __syncthreads();
    }
    fft_line_ct<+1, R, LGZ>(v, t, tw, S, idx);
    if constexpr (TST) {
      put(S);
      if (threadIdx.x == 0) {
        store_field(S, f);
        if (f > 0) {   // region f-1's store has read its source: a_{f-1} again, for the k^2 part
          bulk_wait_read<1>();
          load_field(f - 1, 3 + f - 1);
        }
      }
    } else {
      C* out = reinterpret_cast<C*>(w.at(f));
#pragma unroll
      for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
      // region f is free once every thread is past the transform's last exchange
      // read: a_f again, for the k^2 part, by tensor copies behind the stores
      fence_proxy_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) load_field(f, 3 + f);
    }
  }
  for (int c3 = 0; c3 < 3; ++c3) {
    E* S = c3 == 0 ? S0 : (c3 == 1 ? S1 : S2);
    wait(3 + c3);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int z = t + i * T;
      const int lim = valid ? tb.xcut[(size_t)z * g.ny + y] : 0;
      E av = kept(S, z, lim);
      const R kzs = tb.fkzs[z];
#pragma unroll
      for (int c = 0; c < W; ++c) {
        const R k2 = (kxs[c] + kys) + kzs;
        const C q = col(av, c);
        col(av, c) = C{k2 * q.x, k2 * q.y};
      }
      v[i] = av;
    }
    __syncthreads();   // every thread holds its inputs before the exchanges overwrite the region
    fft_line_ct<+1, R, LGZ>(v, t, tw, S, idx);
    if constexpr (TST) {
      put(S);
      if (threadIdx.x == 0) {
        store_field(S, 3 + c3);
        if (c3 == 0) {   // the u_z store has read region 2: a_2 again
          bulk_wait_read<1>();
          load_field(2, 5);
        }
      }
    } else {
      C* out = reinterpret_cast<C*>(w.at(3 + c3));
#pragma unroll
      for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
    }
  }
  // the stores read the regions until they complete: the block (and its
  // shared memory) stays until the issuing thread has seen them complete
  if constexpr (TST) {
    if (threadIdx.x == 0) bulk_wait_all();
  }
}

// ---------------------------------------------------------------------------
// Pass 1 as a persistent, software-pipelined kernel (z_split = 3): each block
// walks the tile list (member-major for a batched launch) with the same three
// shared regions as k_zinv_curl.  A tile's inputs a_0..a_2 arrive by
// asynchronous copies into regions 0..2; each region, once the k^2 transform
// of the previous tile has finished with it, receives the next tile's input
// column, so neither the curl's loads nor the k^2 part's reloads stall the
// block.  Same columns, pruning and results as k_zinv_curl.
// ---------------------------------------------------------------------------
template <typename R, int LGZ>
__global__ void __launch_bounds__(max_threads<R>() / zcols<R>())
k_zinv_curl_pf(Ptr6 a, Ptr6 w, DevTables<R> tb, Geom g, int lgTX, int pruned, const int32_t* __restrict__ tiles,
               int per_member, int ntx, long long nitems, long long mstride) {
  using C = Cplx<R>;
  constexpr int W = zcols<R>();
  using E = ColT<R, W>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  constexpr int T = 1 << (LGZ - 3);
  const size_t plane = (size_t)g.ny * g.nhp;
  const int reg = strided_rows(1 << LGZ) * TP;
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  auto region = [&](int c) { return sm + c * reg; };
  // item -> the tile's row y, first column X0, column limit and element base
  auto locate = [&](long long item, int& y, int& X0, int& ylim, size_t& base) {
    const long long mem = item / per_member;
    const int ti = (int)(item - mem * per_member);
    int tile;
    if (pruned) {
      tile = tiles[2 * ti];
      y = tiles[2 * ti + 1];
    } else {
      tile = ti % ntx;
      y = ti / ntx;
    }
    X0 = tile * TX + W * xp;
    ylim = pruned ? tb.xcut[y] : g.nh;
    base = (size_t)y * g.nhp + (X0 < ylim ? X0 : 0) + member_offset(mstride, (unsigned)mem);
  };
  auto prefetch = [&](long long item, int c3) {
    int y, X0, ylim;
    size_t base;
    locate(item, y, X0, ylim, base);
    const C* ac = reinterpret_cast<const C*>(a.at(c3));
    E* Sd = region(c3);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int z = t + i * T;
      const int lim = X0 < ylim ? (pruned ? tb.xcut[(size_t)z * g.ny + y] : g.nh) : 0;
      load_cols_async<R, W>(Sd + idx(z), ac, (size_t)z * plane + base, X0, lim);
    }
  };
  long long item = blockIdx.x;
  if (item < nitems) {
    prefetch(item, 0);
    prefetch(item, 1);
    prefetch(item, 2);
  }
  cp_async_commit();
  for (; item < nitems; item += gridDim.x) {
    const bool more = item + gridDim.x < nitems;
    int y, X0, ylim;
    size_t base;
    locate(item, y, X0, ylim, base);
    R kx[W], kxs[W];
#pragma unroll
    for (int c = 0; c < W; ++c) {
      const bool in = X0 + c < ylim;
      kx[c] = in ? tb.fkx[X0 + c] : (R)0;
      kxs[c] = in ? tb.fkxs[X0 + c] : (R)0;
    }
    const R ky = tb.fky[y], kys = tb.fkys[y];
    cp_async_wait(0);   // this thread's copies of the tile's inputs have landed
    E v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int z = t + i * T;
      E ax = region(0)[idx(z)], ay = region(1)[idx(z)], az = region(2)[idx(z)];
      const R kz = tb.fkz[z];
      E ux, uy, uz;
#pragma unroll
      for (int c = 0; c < W; ++c) {
        const C px = col(ax, c), py = col(ay, c), pz = col(az, c);
        col(ux, c) = C{-ky * pz.y + kz * py.y, ky * pz.x - kz * py.x};
        col(uy, c) = C{-kz * px.y + kx[c] * pz.y, kz * px.x - kx[c] * pz.x};
        col(uz, c) = C{-kx[c] * py.y + ky * px.y, kx[c] * py.x - ky * px.x};
      }
      v[i] = ux;
      region(1)[idx(z)] = uy;   // this thread's own slots, read just above
      region(2)[idx(z)] = uz;
    }
    __syncthreads();   // every thread has read its inputs before the exchanges overwrite region 0
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
      E* S = region(f);
      if (f > 0) {
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
        __syncthreads();
      }
      fft_line_ct<+1, R, LGZ>(v, t, tw, S, idx);
      prefetch(item, f);   // the k^2 part's input a_f, into the region the transform has finished with
      cp_async_commit();
      C* out = reinterpret_cast<C*>(w.at(f));
#pragma unroll
      for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
    }
#pragma unroll 1
    for (int c3 = 0; c3 < 3; ++c3) {
      E* S = region(c3);
      cp_async_wait(2);   // a_c3 has landed (the two later groups may still be in flight)
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int z = t + i * T;
        E av = S[idx(z)];
        const R kzs = tb.fkzs[z];
#pragma unroll
        for (int c = 0; c < W; ++c) {
          const R k2 = (kxs[c] + kys) + kzs;
          const C q = col(av, c);
          col(av, c) = C{k2 * q.x, k2 * q.y};
        }
        v[i] = av;
      }
      __syncthreads();
      fft_line_ct<+1, R, LGZ>(v, t, tw, S, idx);
      if (more) prefetch(item + gridDim.x, c3);   // the next tile's a_c3
      cp_async_commit();
      C* out = reinterpret_cast<C*>(w.at(3 + c3));
#pragma unroll
      for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
    }
    if constexpr (LGZ == 3) __syncthreads();   // one-stage transforms have no barrier of their own
  }
  cp_async_wait(0);   // nothing in flight at exit
}

// ---------------------------------------------------------------------------
// Pass 1's w = k^2 a on its own (nlt.f90:26-40): per (x-tile, y) column block
// of the tile list and field f = blockIdx.y, the scaled field's inverse z
// transform with one shared region, so that more blocks are resident than in
// the three-region curl kernel.  Same columns, pruning and output as the
// k^2 half of k_zinv_curl.
// ---------------------------------------------------------------------------
template <typename R, int LGZ>
__global__ void __launch_bounds__(kSpassThreads, sizeof(R) == 8 ? 2 : 3)
k_zk2(Ptr6 a, Ptr6 w, DevTables<R> tb, Geom g, int lgTX, int pruned, const int32_t* __restrict__ tiles,
      long long mstride) {
  using C = Cplx<R>;
  constexpr int W = zcols<R>();
  using E = ColT<R, W>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  // grid: (tiles, field, member) pruned; (tiles, field, member * ny + y) full
  int tile = blockIdx.x, y = blockIdx.z % g.ny;
  unsigned mem = blockIdx.z / g.ny;
  if (pruned) {
    tile = tiles[2 * blockIdx.x];
    y = tiles[2 * blockIdx.x + 1];
    mem = blockIdx.z;
  }
  const int f = blockIdx.y;
  const int X0 = tile * TX + W * xp;
  const int ylim = pruned ? tb.xcut[y] : g.nh;
  const bool valid = X0 < ylim;
  constexpr int T = 1 << (LGZ - 3);
  const size_t plane = (size_t)g.ny * g.nhp;
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0) + member_offset(mstride, mem);
  const StridedIdxLg idx{lgTP, xp};
  R kxs[W];
#pragma unroll
  for (int c = 0; c < W; ++c) kxs[c] = X0 + c < ylim ? tb.fkxs[X0 + c] : (R)0;
  const R kys = tb.fkys[y];
  const C* ac = reinterpret_cast<const C*>(a.at(f));
  E v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int z = t + i * T;
    const int lim = valid ? (pruned ? tb.xcut[(size_t)z * g.ny + y] : g.nh) : 0;
    E av = load_cols<R, W>(ac, (size_t)z * plane + base, X0, lim);
    const R kzs = tb.fkzs[z];
#pragma unroll
    for (int c = 0; c < W; ++c) {
      const R k2 = (kxs[c] + kys) + kzs;
      const C q = col(av, c);
      col(av, c) = C{k2 * q.x, k2 * q.y};
    }
    v[i] = av;
  }
  fft_line_ct<+1, R, LGZ>(v, t, reinterpret_cast<const C*>(tb.twz), sm, idx);
  C* out = reinterpret_cast<C*>(w.at(3 + f));
#pragma unroll
  for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
}

// ---------------------------------------------------------------------------
// Pass 1 in one shared region: each of the six output lines (u = i k x a and
// w = k^2 a) is formed from the input columns read again (after the first
// read, from L2) instead of being parked in shared memory, so that a block
// needs a third of the shared memory of k_zinv_curl and, with one or two
// input fields live at a time, fewer registers: three resident blocks of 256
// threads for FP32 instead of two.  Same columns, pruning and output, the
// same expressions per element.
// ---------------------------------------------------------------------------
template <typename R, int LGZ>
__global__ void __launch_bounds__(kSpassThreads, sizeof(R) == 8 ? 2 : 3)
k_zinv_curl1(Ptr6 a, Ptr6 w, DevTables<R> tb, Geom g, int lgTX, int pruned, const int32_t* __restrict__ tiles,
             long long mstride) {
  using C = Cplx<R>;
  constexpr int W = zcols<R>();
  using E = ColT<R, W>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  int tile = blockIdx.x, y = blockIdx.y;
  if (pruned) {
    tile = tiles[2 * blockIdx.x];
    y = tiles[2 * blockIdx.x + 1];
  }
  const int X0 = tile * TX + W * xp;
  const int ylim = pruned ? tb.xcut[y] : g.nh;
  const bool valid = X0 < ylim;
  constexpr int T = 1 << (LGZ - 3);
  const size_t plane = (size_t)g.ny * g.nhp;
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0) + member_offset(mstride, pruned ? blockIdx.y : blockIdx.z);
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  R kx[W], kxs[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    const bool in = X0 + c < ylim;
    kx[c] = in ? tb.fkx[X0 + c] : (R)0;
    kxs[c] = in ? tb.fkxs[X0 + c] : (R)0;
  }
  const R ky = tb.fky[y], kys = tb.fkys[y];
  E v[8];
#pragma unroll 1
  for (int f = 0; f < 6; ++f) {
    // the fields output f reads: u_0 <- (a1, a2), u_1 <- (a0, a2), u_2 <- (a0, a1); w_c <- a_c
    const C* p1 = reinterpret_cast<const C*>(a.at(f < 3 ? (f == 0 ? 1 : 0) : f - 3));
    const C* p2 = reinterpret_cast<const C*>(a.at(f == 2 ? 1 : 2));
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int z = t + i * T;
      const int lim = valid ? (pruned ? tb.xcut[(size_t)z * g.ny + y] : g.nh) : 0;
      const size_t o = (size_t)z * plane + base;
      E q1 = load_cols<R, W>(p1, o, X0, lim);
      E r;
      if (f < 3) {
        E q2 = load_cols<R, W>(p2, o, X0, lim);
        const R kz = tb.fkz[z];
#pragma unroll
        for (int c = 0; c < W; ++c) {
          const C b1 = col(q1, c), b2 = col(q2, c);
          if (f == 0) {          // (py, pz) = (b1, b2)
            col(r, c) = C{-ky * b2.y + kz * b1.y, ky * b2.x - kz * b1.x};
          } else if (f == 1) {   // (px, pz) = (b1, b2)
            col(r, c) = C{-kz * b1.y + kx[c] * b2.y, kz * b1.x - kx[c] * b2.x};
          } else {               // (px, py) = (b1, b2)
            col(r, c) = C{-kx[c] * b2.y + ky * b1.y, kx[c] * b2.x - ky * b1.x};
          }
        }
      } else {
        const R kzs = tb.fkzs[z];
#pragma unroll
        for (int c = 0; c < W; ++c) {
          const R k2 = (kxs[c] + kys) + kzs;
          const C qq = col(q1, c);
          col(r, c) = C{k2 * qq.x, k2 * qq.y};
        }
      }
      v[i] = r;
    }
    // the previous line's last reads of sm precede the final barrier of its
    // transform, so the scratch is free again here
    fft_line_ct<+1, R, LGZ>(v, t, tw, sm, idx);
    C* out = reinterpret_cast<C*>(w.at(f));
#pragma unroll
    for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
  }
}

// ---------------------------------------------------------------------------
// Strided (y or z) transform of up to six fields, in place.  blockIdx.z picks
// the field, blockIdx.y the outer index (z for a y pass, y for a z pass).
// ---------------------------------------------------------------------------
// At most 256 threads per block; for FP32 five resident blocks (48
// registers), which hides more load latency than four blocks of 64 registers
// (measured at 512^3: inverse y pass 1.04 ms against 1.11 ms).
template <typename R> constexpr int spass_min_blocks() { return sizeof(R) == 8 ? 2 : 5; }

template <typename R, int SIGN, int LGL>
__global__ void __launch_bounds__(kSpassThreads, spass_min_blocks<R>())
k_spass(Ptr6 f, Geom g, const void* twv, long long ls, long long os, int lgTX, int xlim,
        int ymask, const int32_t* __restrict__ xcut0, int nf, long long mstride) {
  using C = Cplx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int TX = 1 << lgTX;
  const int x = threadIdx.x & (TX - 1), t = threadIdx.x >> lgTX;
  const int X = blockIdx.x * TX + x;
  const bool valid = X < xlim;
  constexpr int T = 1 << (LGL - 3);
  // blockIdx.z = member * nf + field
  C* p = reinterpret_cast<C*>(f.at(blockIdx.z % nf));
  const size_t base = (size_t)blockIdx.y * (size_t)os + (valid ? X : 0) + member_offset(mstride, blockIdx.z / nf);
  const StridedIdxLg idx{lgTX, x};
  C v[8];
  // ymask 1 (pruned inverse y pass): only (X, y) with X < xcut0[y] hold data;
  // ymask 2 (pruned forward y pass): only those are stored.
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int e = t + i * T;
    const bool ld = valid && (ymask != 1 || X < xcut0[e]);
    v[i] = ld ? p[base + (size_t)e * (size_t)ls] : C{0, 0};
  }
  fft_line_ct<SIGN, R, LGL>(v, t, reinterpret_cast<const C*>(twv), sm, idx);
  if (valid) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = t + i * T;
      if (ymask != 2 || X < xcut0[e]) p[base + (size_t)e * (size_t)ls] = v[i];
    }
  }
}

// ---------------------------------------------------------------------------
// The strided transform with two adjacent x columns per thread (FP32): one
// 16-byte load or store per position, the stage twiddles and index
// arithmetic shared by both columns, twice the bytes in flight per thread.
// Block: (L/8) x TP threads for a tile of 2 TP columns; the shared tile is
// [rows][TP] column pairs with the y/z padding rows.  Column X0 = 2 (tile TP
// + xp); a pair straddling xlim or the pruning cut moves element by element.
// ---------------------------------------------------------------------------
// The inverse y pass (six fields, loads masked by the truncation) runs best
// at 4 resident blocks (64 registers, small spills), the forward one at 3
// (80 registers): 0.90 / 0.36 ms at 512^3.
template <int SIGN, int LGL>
__global__ void __launch_bounds__(kSpassThreads, SIGN > 0 ? 4 : 3)
k_spass2(Ptr6 f, Geom g, const void* twv, long long ls, long long os, int lgTP, int xlim, int ymask,
         const int32_t* __restrict__ xcut0, int nf, long long mstride) {
  using C = float2;
  using E = CPair<float>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  const int X0 = 2 * (blockIdx.x * TP + xp);
  constexpr int T = 1 << (LGL - 3);
  // blockIdx.z = member * nf + field
  C* p = reinterpret_cast<C*>(f.at(blockIdx.z % nf));
  const size_t base = (size_t)blockIdx.y * (size_t)os + (X0 < xlim ? X0 : 0) + member_offset(mstride, blockIdx.z / nf);
  const StridedIdxLg idx{lgTP, xp};
  E v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int e = t + i * T;
    const int cut = ymask == 1 ? min(xlim, xcut0[e]) : xlim;
    const C* src = p + base + (size_t)e * (size_t)ls;
    if (X0 + 1 < cut) {
      v[i] = *reinterpret_cast<const E*>(src);
    } else {
      v[i].a = X0 < cut ? src[0] : C{0, 0};
      v[i].b = C{0, 0};
    }
  }
  fft_line_ct<SIGN, float, LGL>(v, t, reinterpret_cast<const C*>(twv), sm, idx);
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int e = t + i * T;
    const int cut = ymask == 2 ? min(xlim, xcut0[e]) : xlim;
    C* dst = p + base + (size_t)e * (size_t)ls;
    if (X0 + 1 < cut) {
      *reinterpret_cast<E*>(dst) = v[i];
    } else if (X0 < cut) {
      dst[0] = v[i].a;
    }
  }
}

// ---------------------------------------------------------------------------
// The FP32 strided transform as a persistent pass: each block walks tiles
// (x-tile fastest, then the outer index, field and member) and double-buffers
// them in shared memory; the next tile's columns are copied asynchronously
// (cp.async, zero-filled where the truncation masks them) while the current
// tile is transformed, so every block keeps a tile of loads in flight instead
// of stalling on them between transforms.  Same columns, masks and results as
// k_spass2.
// ---------------------------------------------------------------------------
template <int SIGN, int LGL>
__global__ void __launch_bounds__(kSpassThreads, 3)
k_spass2_pf(Ptr6 f, Geom g, const void* twv, long long ls, long long os, int lgTP, int xlim, int ymask,
            const int32_t* __restrict__ xcut0, int nf, long long mstride, int ntx, int nouter,
            long long nitems) {
  using C = float2;
  using E = CPair<float>;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  constexpr int T = 1 << (LGL - 3);
  const int stage_elems = strided_rows(1 << LGL) * TP;
  E* const st0 = reinterpret_cast<E*>(smraw);
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(twv);
  // item -> (field pointer, element base, first column)
  auto locate = [&](long long item, C*& p, size_t& base, int& X0) {
    const int tx = (int)(item % ntx);
    const long long r = item / ntx;
    const int outer = (int)(r % nouter);
    const int fz = (int)(r / nouter);   // member * nf + field
    X0 = 2 * (tx * TP + xp);
    p = reinterpret_cast<C*>(f.at(fz % nf));
    base = (size_t)outer * (size_t)os + (X0 < xlim ? X0 : 0) + member_offset(mstride, fz / nf);
  };
  auto prefetch = [&](long long item, E* S) {
    C* p;
    size_t base;
    int X0;
    locate(item, p, base, X0);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = t + i * T;
      const int cut = ymask == 1 ? min(xlim, xcut0[e]) : xlim;
      const int n = X0 + 1 < cut ? 16 : (X0 < cut ? 8 : 0);
      cp_async<16>(S + idx(e), p + base + (size_t)e * (size_t)ls, n);
    }
  };
  long long item = blockIdx.x;
  if (item < nitems) prefetch(item, st0);
  cp_async_commit();
  for (int it = 0; item < nitems; item += gridDim.x, ++it) {
    E* S = st0 + (it & 1) * stage_elems;
    // the other stage was last used by the previous tile, whose final
    // barrier every thread has passed
    if (item + gridDim.x < nitems) prefetch(item + gridDim.x, st0 + ((it + 1) & 1) * stage_elems);
    cp_async_commit();
    cp_async_wait(1);   // this thread's copies of the current tile have landed
    E v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
    __syncthreads();    // every thread holds its inputs before the exchanges overwrite the stage
    fft_line_ct<SIGN, float, LGL>(v, t, tw, S, idx);
    C* p;
    size_t base;
    int X0;
    locate(item, p, base, X0);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = t + i * T;
      const int cut = ymask == 2 ? min(xlim, xcut0[e]) : xlim;
      C* dst = p + base + (size_t)e * (size_t)ls;
      if (X0 + 1 < cut) {
        *reinterpret_cast<E*>(dst) = v[i];
      } else if (X0 < cut) {
        dst[0] = v[i].a;
      }
    }
    if constexpr (LGL == 3) __syncthreads();   // no barrier in a one-stage transform: free the stage
  }
  cp_async_wait(0);   // nothing in flight at exit
}

// ---------------------------------------------------------------------------
// Pass 3: x transforms with the cross product fused in.  A block holds P
// pairs of rows; each pair uses three groups of N/8 threads.  Inverse: the
// half spectra of fields (2q, 2q+1) of one row are packed as X1 + i X2 into
// one complex line (q = 0..2), so one inverse complex FFT yields both real
// rows.  Forward: (c_x + i c_y) of row 0, of row 1 and (c_z row 0 + i c_z
// row 1) are transformed and split with X1 = (Y_k + conj Y_{N-k})/2,
// X2 = (Y_k - conj Y_{N-k})/(2i).
// ---------------------------------------------------------------------------
// Half-spectrum entries at kx >= xa are zero (pruned pipeline) and are not read.
// Z_e = X1_e + i X2_e (e < N/2), conj(X1_{N-e}) + i conj(X2_{N-e}) (e > N/2);
// at e = 0 and N/2 only the real parts enter (numpy irfft convention).
template <typename R>
__device__ __forceinline__ Cplx<R> pack_c2r(const Cplx<R>* __restrict__ X1,
                                            const Cplx<R>* __restrict__ X2, int e, int N, int xa) {
  using C = Cplx<R>;
  const int h = N >> 1;
  const bool hi = e > h;
  const int k = hi ? N - e : e;
  if (k >= xa) return C{0, 0};
  C a = X1[k], b = X2[k];
  if (k == 0 || k == h) {
    a.y = 0;
    b.y = 0;
  }
  const R sg = hi ? (R)-1 : (R)1;
  return C{a.x - sg * b.y, sg * a.y + b.x};
}

// The same packing for position e = t + I N/8 of thread t of a line's N/8
// threads, with the position's half and special cases resolved at compile
// time: I < 4 lies below N/2 (k = e; e = 0 only for I = 0, t = 0), I = 4 is
// N/2 + t (k = N/2 - t; the Nyquist entry for t = 0), I > 4 lies above
// (k = N - e).  Equal to pack_c2r(X1, X2, e, N, xa).
template <typename R, int I, int N>
__device__ __forceinline__ Cplx<R> pack_c2r_at(const Cplx<R>* __restrict__ X1, const Cplx<R>* __restrict__ X2,
                                               int t, int xa) {
  using C = Cplx<R>;
  constexpr int T = N / 8, H = N / 2;
  if constexpr (I < 4) {
    const int k = t + I * T;
    if (k >= xa) return C{0, 0};
    C a = X1[k], b = X2[k];
    if constexpr (I == 0) {
      if (t == 0) { a.y = 0; b.y = 0; }
    }
    return C{a.x - b.y, a.y + b.x};
  } else if constexpr (I == 4) {
    const int k = H - t;
    if (k >= xa) return C{0, 0};
    C a = X1[k], b = X2[k];
    if (t == 0) { a.y = 0; b.y = 0; return C{a.x - b.y, a.y + b.x}; }
    return C{a.x + b.y, b.x - a.y};
  } else {
    const int k = (8 - I) * T - t;
    if (k >= xa) return C{0, 0};
    const C a = X1[k], b = X2[k];
    return C{a.x + b.y, b.x - a.y};
  }
}

// Calls f(std::integral_constant<int, I>) for I = 0..7: a loop over the 8
// positions of a thread whose index is a compile-time constant in the body.
template <typename F>
__device__ __forceinline__ void for8(F&& f) {
  f(std::integral_constant<int, 0>{}); f(std::integral_constant<int, 1>{});
  f(std::integral_constant<int, 2>{}); f(std::integral_constant<int, 3>{});
  f(std::integral_constant<int, 4>{}); f(std::integral_constant<int, 5>{});
  f(std::integral_constant<int, 6>{}); f(std::integral_constant<int, 7>{});
}

template <typename R>
__device__ __forceinline__ Cplx<R> split_r2c(Cplx<R> a, Cplx<R> b, bool first, R s) {
  using C = Cplx<R>;
  return first ? C{(a.x + b.x) * s, (a.y - b.y) * s} : C{(a.y + b.y) * s, (b.x - a.x) * s};
}

template <typename R, int LGN>
__global__ void __launch_bounds__(xcross_threads<LGN>(), (xcross_min_blocks<R, LGN>()))
k_xcross(Ptr6 w, Geom g, const void* twv, int P, R shalf, int xa, long long mstride) {
  using C = Cplx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int N = 1 << LGN, lgN = LGN, lgT = LGN - 3, T = 1 << lgT;
  constexpr int LP = N;
  const int gid = threadIdx.x >> lgT, t = threadIdx.x & (T - 1);
  const int p = gid / 3, q = gid - 3 * p;
  const size_t pair = (size_t)blockIdx.x * P + p;
  const C* tw = reinterpret_cast<const C*>(twv);
  const size_t nhp = g.nhp;
  const size_t mo = member_offset(mstride, blockIdx.y);   // batched launch: member blockIdx.y
  C v[8];
  // inverse: rows 0 and 1 of the pair, field pair q
#pragma unroll 1
  for (int r = 0; r < 2; ++r) {
    const size_t row = 2 * pair + r;
    const C* X1 = reinterpret_cast<const C*>(w.at(2 * q)) + mo + row * nhp;
    const C* X2 = reinterpret_cast<const C*>(w.at(2 * q + 1)) + mo + row * nhp;
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = pack_c2r<R>(X1, X2, t + i * T, N, xa);
    const SwzIdx idx{(p * 6 + r * 3 + q) * LP};
    fft_line_ct<+1, R, LGN>(v, t, tw, sm, idx);
#pragma unroll
    for (int i = 0; i < 8; ++i) sm[idx(t + i * T)] = v[i];
  }
  __syncthreads();
  // u x w per point of both rows (produ.f90:14-16); u = (z0.x, z0.y, z1.x),
  // w = (z1.y, z2.x, z2.y) for row 0 and (z3..z5) for row 1.
  for (int n = threadIdx.x; n < P * N; n += blockDim.x) {
    const int pp = n >> lgN, e = n & (N - 1);
    const int o = pp * 6 * LP + swz(e);
    const C z0 = sm[o], z1 = sm[o + LP], z2 = sm[o + 2 * LP];
    const C z3 = sm[o + 3 * LP], z4 = sm[o + 4 * LP], z5 = sm[o + 5 * LP];
    const R c0x = z0.y * z2.y - z1.x * z2.x;
    const R c0y = z1.x * z1.y - z0.x * z2.y;
    const R c0z = z0.x * z2.x - z0.y * z1.y;
    const R c1x = z3.y * z5.y - z4.x * z5.x;
    const R c1y = z4.x * z4.y - z3.x * z5.y;
    const R c1z = z3.x * z5.x - z3.y * z4.y;
    sm[o] = C{c0x, c0y};
    sm[o + 3 * LP] = C{c1x, c1y};
    sm[o + LP] = C{c0z, c1z};
  }
  __syncthreads();
  {
    const int line = p * 6 + (q == 0 ? 0 : (q == 1 ? 3 : 1));
    const SwzIdx idx{line * LP};
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = sm[idx(t + i * T)];
    __syncthreads();
    fft_line_ct<-1, R, LGN>(v, t, tw, sm, idx);
#pragma unroll
    for (int i = 0; i < 8; ++i) sm[idx(t + i * T)] = v[i];
  }
  __syncthreads();
  // Group q of pair p writes field q (c_x, c_y, c_z) of both rows; kx >= xa
  // is truncated later (pruned) or xa = nh.
  {
    const int lineA = p * 6 + (q == 2 ? 1 : 0), lineB = p * 6 + (q == 2 ? 1 : 3);
    C* out = reinterpret_cast<C*>(w.at(q));
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int o = (r == 0 ? lineA : lineB) * LP;
      const bool first = (q == 0) || (q == 2 && r == 0);
      C* orow = out + mo + (2 * pair + r) * nhp;
      for (int k = t; k < xa; k += T) {
        const int kb = (N - k) & (N - 1);
        const C a = sm[o + swz(k)], b = sm[o + swz(kb)];
        orow[k] = split_r2c<R>(a, b, first, shalf);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Pass 3, register-resident form: one group of N/8 threads owns a whole pair
// of rows.  It runs the three packed inverse transforms of row 0 one after the
// other, keeping the first two results in registers, so that u x w is formed
// in registers in the natural order the last Stockham stage leaves; the
// packed line c_x + i c_y goes straight into the forward transform, c_z waits
// in registers for row 1 and is packed with it.  Shared memory is used only
// for the transforms' own exchanges and for the r2c split (which needs
// Z[k] and Z[N-k]): 41 N line accesses per row pair instead of 61 N.  Groups
// synchronise on their own named barrier when they fill whole warps.
// ---------------------------------------------------------------------------
template <typename R> constexpr int xfused_threads() { return sizeof(R) == 8 ? 128 : 256; }

template <typename R, int LGN>
__global__ void __launch_bounds__(xfused_threads<R>(), 2)
k_xfused(Ptr6 w, Geom g, const void* twv, R shalf, int xa, long long mstride) {
  using C = Cplx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int N = 1 << LGN, T = N / 8;
  constexpr int LP = N;
  const int grp = threadIdx.x >> (LGN - 3), t = threadIdx.x & (T - 1);
  const int P = blockDim.x >> (LGN - 3);
  const size_t pair = (size_t)blockIdx.x * P + grp;
  const C* tw = reinterpret_cast<const C*>(twv);
  const size_t nhp = g.nhp;
  const size_t mo = member_offset(mstride, blockIdx.y);   // batched launch: member blockIdx.y
  const SwzIdx idx{grp * LP};
  C* line = sm + grp * LP;
  C v[8], z0[8], z1[8];
  R cz0[8];
  auto run = [&](auto sync) {
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
      const size_t row = 2 * pair + r;
#pragma unroll 1
      for (int q = 0; q < 3; ++q) {
        const C* X1 = reinterpret_cast<const C*>(w.at(2 * q)) + mo + row * nhp;
        const C* X2 = reinterpret_cast<const C*>(w.at(2 * q + 1)) + mo + row * nhp;
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = pack_c2r<R>(X1, X2, t + i * T, N, xa);
        fft_line_ct<+1, R, LGN>(v, t, tw, sm, idx, sync);
        if (q == 0) {
#pragma unroll
          for (int i = 0; i < 8; ++i) z0[i] = v[i];
        } else if (q == 1) {
#pragma unroll
          for (int i = 0; i < 8; ++i) z1[i] = v[i];
        }
      }
      // u = (z0.x, z0.y, z1.x), w = (z1.y, v.x, v.y) (produ.f90:14-16)
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const R cx = z0[i].y * v[i].y - z1[i].x * v[i].x;
        const R cy = z1[i].x * z1[i].y - z0[i].x * v[i].y;
        const R cz = z0[i].x * v[i].x - z0[i].y * z1[i].y;
        if (r == 0) {
          cz0[i] = cz;
        } else {
          z1[i] = C{cz0[i], cz};
        }
        v[i] = C{cx, cy};
      }
      // forward c_x + i c_y of this row -> fields 0 and 1
#pragma unroll 1
      for (int pass = 0; pass < (r == 0 ? 1 : 2); ++pass) {
        if (pass == 1) {
#pragma unroll
          for (int i = 0; i < 8; ++i) v[i] = z1[i];
        }
        fft_line_ct<-1, R, LGN>(v, t, tw, sm, idx, sync);
#pragma unroll
        for (int i = 0; i < 8; ++i) sm[idx(t + i * T)] = v[i];
        sync();
        // pass 0: Z = c_x + i c_y of row r; pass 1: Z = c_z(row 0) + i c_z(row 1)
        C* oa = reinterpret_cast<C*>(pass == 0 ? w.p[0] : w.p[2]) + mo + (pass == 0 ? row : 2 * pair) * nhp;
        C* ob = reinterpret_cast<C*>(pass == 0 ? w.p[1] : w.p[2]) + mo + (pass == 0 ? row : 2 * pair + 1) * nhp;
        for (int k = t; k < xa; k += T) {
          const int kb = (N - k) & (N - 1);
          const C a = line[swz(k)], b = line[swz(kb)];
          oa[k] = split_r2c<R>(a, b, true, shalf);
          ob[k] = split_r2c<R>(a, b, false, shalf);
        }
        sync();
      }
    }
  };
  if constexpr (T >= 32) {
    run(NamedSync{1 + grp, T});
  } else {
    run(BlockSync{});
  }
}

// ---------------------------------------------------------------------------
// Pass 3 with the three lines of a row transformed together: one group of N/8
// threads owns a pair of rows; the three packed inverse lines of a row are one
// CTrip transform (shared twiddles, index arithmetic and barriers; three
// interleaved dependency chains), kept as three planes of shared memory.  u x w
// is formed in registers; c_x + i c_y of row 0 waits in registers until the
// three forward lines (c_x + i c_y of rows 0 and 1, c_z(row 0) + i c_z(row 1))
// are one CTrip transform.  3 transform calls per row pair instead of 9.
// ---------------------------------------------------------------------------
template <typename R> constexpr int xbatch_threads() { return sizeof(R) == 8 ? 128 : 256; }

// PARK: row 0's products wait in a shared region (N complex + N real per
// group) instead of registers, for 3 resident blocks instead of 2.
template <typename R, int LGN, bool PARK = false>
__global__ void __launch_bounds__(xbatch_threads<R>(), PARK ? 3 : 2)
k_xbatch(Ptr6 w, Geom g, const void* twv, R shalf, int xa, long long mstride) {
  using C = Cplx<R>;
  using E = CTrip<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int N = 1 << LGN, T = N / 8, LP = N;
  const int grp = threadIdx.x >> (LGN - 3), t = threadIdx.x & (T - 1);
  const int P = blockDim.x >> (LGN - 3);
  const size_t pair = (size_t)blockIdx.x * P + grp;
  const C* tw = reinterpret_cast<const C*>(twv);
  const size_t nhp = g.nhp;
  const size_t mo = member_offset(mstride, blockIdx.y);   // batched launch: member blockIdx.y
  C* lines = sm + (size_t)grp * 3 * LP;
  const TripMem<R, SwzIdx> mem{lines, SwzIdx{0}, LP};
  E v[8];
  C a0[PARK ? 1 : 8];
  R cz0[PARK ? 1 : 8];
  C* park_a = sm + (size_t)3 * P * LP + (size_t)grp * LP;
  R* park_z = reinterpret_cast<R*>(sm + (size_t)4 * P * LP) + (size_t)grp * LP;
  auto run = [&](auto sync) {
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
      const size_t row = 2 * pair + r;
      const size_t ro = mo + row * nhp;
      for8([&](auto I) {
        v[I].a = pack_c2r_at<R, I, N>(reinterpret_cast<const C*>(w.p[0]) + ro,
                                      reinterpret_cast<const C*>(w.p[1]) + ro, t, xa);
        v[I].b = pack_c2r_at<R, I, N>(reinterpret_cast<const C*>(w.p[2]) + ro,
                                      reinterpret_cast<const C*>(w.p[3]) + ro, t, xa);
        v[I].c = pack_c2r_at<R, I, N>(reinterpret_cast<const C*>(w.p[4]) + ro,
                                      reinterpret_cast<const C*>(w.p[5]) + ro, t, xa);
      });
      fft_line_mem<+1, R, LGN, (sizeof(R) == 4 && !PARK)>(v, t, tw, mem, sync);
      // u = (z0.x, z0.y, z1.x), w = (z1.y, z2.x, z2.y) (produ.f90:14-16)
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const C z0 = v[i].a, z1 = v[i].b, z2 = v[i].c;
        const R cx = z0.y * z2.y - z1.x * z2.x;
        const R cy = z1.x * z1.y - z0.x * z2.y;
        const R cz = z0.x * z2.x - z0.y * z1.y;
        if constexpr (PARK) {
          const int e = t + i * T;   // each thread reads back only its own positions
          if (r == 0) {
            park_a[e] = C{cx, cy};
            park_z[e] = cz;
          } else {
            v[i] = E{park_a[e], C{cx, cy}, C{park_z[e], cz}};
          }
        } else if (r == 0) {
          a0[i] = C{cx, cy};
          cz0[i] = cz;
        } else {
          v[i] = E{a0[i], C{cx, cy}, C{cz0[i], cz}};
        }
      }
    }
    // forward: planes 0, 1, 2 = c_x + i c_y of rows 0 and 1, c_z(0) + i c_z(1)
    fft_line_mem<-1, R, LGN, (sizeof(R) == 4 && !PARK)>(v, t, tw, mem, sync);
#pragma unroll
    for (int i = 0; i < 8; ++i) mem.st(t + i * T, v[i]);
    sync();
    const size_t row0 = 2 * pair;
    C* f0 = reinterpret_cast<C*>(w.p[0]);
    C* f1 = reinterpret_cast<C*>(w.p[1]);
    C* f2 = reinterpret_cast<C*>(w.p[2]);
    for (int k = t; k < xa; k += T) {
      const int kb = (N - k) & (N - 1);
      const int ia = swz(k), ib = swz(kb);
#pragma unroll
      for (int pl = 0; pl < 3; ++pl) {
        const C a = lines[pl * LP + ia], b = lines[pl * LP + ib];
        C* oa = (pl == 2 ? f2 : f0) + mo + (row0 + (pl == 1 ? 1 : 0)) * nhp;
        C* ob = (pl == 2 ? f2 : f1) + mo + (row0 + (pl == 0 ? 0 : 1)) * nhp;
        oa[k] = split_r2c<R>(a, b, true, shalf);
        ob[k] = split_r2c<R>(a, b, false, shalf);
      }
    }
  };
  if constexpr (T >= 32) {
    run(NamedSync{1 + grp, T});
  } else {
    run(BlockSync{});
  }
}

// The spectral epilogue of pass 5 (nlt.f90:67-81, produ.f90:83-99,
// trunc.f90:14-28, rkstep.f90:30-48 / 86-104) at one thread's own positions
// of a z tile: the transformed fields are in the three shared regions `reg`
// apart, the state b(t) is read from global memory.
// Thread position e = t + i T of the tile is mode z = zmul e + zadd (zmul = 2,
// zadd = r for the half of a cluster pair that owns the modes z = r mod 2;
// T = 2^(LGT - 3) threads per line).
template <typename R, int LGT, int W, typename Idx = StridedIdxLg>
__device__ __forceinline__ void zfwd_epilogue(const ColT<R, W>* __restrict__ sm, int reg, const Idx& idx,
                                              int t, int X0, int y, int ylim, size_t base, size_t plane,
                                              const Ptr6& bc, const Ptr6& out, const DevTables<R>& tb,
                                              const Geom& g, int mode, int pruned, int zmul = 1, int zadd = 0) {
  using C = Cplx<R>;
  using E = ColT<R, W>;
  constexpr int T = 1 << (LGT - 3);
  const R ky = tb.fky[y], kys = tb.fkys[y];
  const C* b0p = reinterpret_cast<const C*>(bc.p[0]);
  const C* b1p = reinterpret_cast<const C*>(bc.p[1]);
  const C* b2p = reinterpret_cast<const C*>(bc.p[2]);
  C* o0 = reinterpret_cast<C*>(out.p[0]);
  C* o1 = reinterpret_cast<C*>(out.p[1]);
  C* o2 = reinterpret_cast<C*>(out.p[2]);
#pragma unroll 2
  for (int i = 0; i < 8; ++i) {
    const int e = t + i * T;
    const int z = zmul * e + zadd;
    const int zlim = tb.xcut[(size_t)z * g.ny + y];      // kept modes of this row: X < zlim
    // columns whose result is written: all of the row's columns, or only the
    // kept ones when pruned (zero outside K in both the state and the result)
    const int wlim = pruned ? zlim : ylim;
    if (X0 >= wlim) continue;
    const size_t o = (size_t)z * plane + base;
    E n0 = sm[idx(e)], n1 = sm[reg + idx(e)], n2 = sm[2 * reg + idx(e)];
    E bb0 = load_cols<R, W>(b0p, o, X0, wlim), bb1 = load_cols<R, W>(b1p, o, X0, wlim),
      bb2 = load_cols<R, W>(b2p, o, X0, wlim);
    const R kz = tb.fkz[z], kzs = tb.fkzs[z];
    const R okz = tb.omega * kz;
    E res0, res1, res2;
#pragma unroll
    for (int c = 0; c < W; ++c) {
      const int X = X0 + c;
      const C b0 = col(bb0, c), b1 = col(bb1, c), b2 = col(bb2, c);
      const C m0 = col(n0, c), m1 = col(n1, c), m2 = col(n2, c);
      // nlt.f90:67-81: a = v + i omega kz b(t)
      const C a0{m0.x - okz * b0.y, m0.y + okz * b0.x};
      const C a1{m1.x - okz * b1.y, m1.y + okz * b1.x};
      const C a2{m2.x - okz * b2.y, m2.y + okz * b2.x};
      const bool zero_mode = (X == 0) && (y == 0) && (z == 0);
      const bool kept = X < zlim;
      const R kxv = X < g.nh ? tb.fkx[X] : (R)0, kxsv = X < g.nh ? tb.fkxs[X] : (R)0;
      const R k2 = (kxsv + kys) + kzs;
      C r0 = a0, r1 = a1, r2 = a2;
      if (!zero_mode) {  // produ.f90:83-99: i k x a / k^2
        const R ik2 = (R)1 / k2;
        const R qx = kxv * ik2, qy = ky * ik2, qz = kz * ik2;
        r0 = C{-qy * a2.y + qz * a1.y, qy * a2.x - qz * a1.x};
        r1 = C{-qz * a0.y + qx * a2.y, qz * a0.x - qx * a2.x};
        r2 = C{-qx * a1.y + qy * a0.y, qx * a1.x - qy * a0.x};
      }
      if (tb.truncate && (zero_mode || !kept)) {  // trunc.f90:14-28
        r0 = C{0, 0}; r1 = C{0, 0}; r2 = C{0, 0};
      }
      if (mode == kNltOnly) {
        col(res0, c) = r0; col(res1, c) = r1; col(res2, c) = r2;
      } else {
        const R e = X >= g.nh ? (R)0
                    : (tb.emk_by_k2 ? tb.emk[(int)k2] : tb.emk[((size_t)z * g.ny + y) * g.nh + X]);
        C s0, s1, s2;
        if (mode == kStage1) {  // rkstep.f90:30-40: c = emk (a + dt2 c)
          const R d = tb.dt2;
          s0 = C{e * (b0.x + d * r0.x), e * (b0.y + d * r0.y)};
          s1 = C{e * (b1.x + d * r1.x), e * (b1.y + d * r1.y)};
          s2 = C{e * (b2.x + d * r2.x), e * (b2.y + d * r2.y)};
        } else {                // rkstep.f90:86-96: a = emk (emk a + dt c)
          const R d = tb.dt;
          s0 = C{e * (e * b0.x + d * r0.x), e * (e * b0.y + d * r0.y)};
          s1 = C{e * (e * b1.x + d * r1.x), e * (e * b1.y + d * r1.y)};
          s2 = C{e * (e * b2.x + d * r2.x), e * (e * b2.y + d * r2.y)};
        }
        if (zero_mode) {        // rkstep.f90:44-48 / 100-104
          s0 = C{0, 0}; s1 = C{0, 0}; s2 = C{0, 0};
        }
        col(res0, c) = s0; col(res1, c) = s1; col(res2, c) = s2;
      }
    }
    store_cols<R, W>(o0, o, X0, wlim, res0);
    store_cols<R, W>(o1, o, X0, wlim, res1);
    store_cols<R, W>(o2, o, X0, wlim, res2);
  }
}

// ---------------------------------------------------------------------------
// Pass 5: forward z transform of three fields, then the spectral epilogue.
// ---------------------------------------------------------------------------
template <typename R, int LGZ>
__global__ void __launch_bounds__(max_threads<R>() / zfwd_cols<R>())
k_zfwd_epi(Ptr6 w, Ptr6 bc, Ptr6 out, DevTables<R> tb, Geom g, int lgTX, int mode, int pruned,
           const int32_t* __restrict__ tiles, Batch<R> bt) {
  using C = Cplx<R>;
  constexpr int W = zfwd_cols<R>();
  using E = ColT<R, W>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  int tile = blockIdx.x, y = blockIdx.y;
  if (pruned) {
    tile = tiles[2 * blockIdx.x];
    y = tiles[2 * blockIdx.x + 1];
  }
  const int X0 = tile * TX + W * xp;
  const int ylim = pruned ? tb.xcut[y] : g.nh;
  const bool valid = X0 < ylim;
  constexpr int T = 1 << (LGZ - 3);
  const size_t plane = (size_t)g.ny * g.nhp;
  const unsigned mem = pruned ? blockIdx.y : blockIdx.z;
  member_tables(bt, mem, tb);
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0) + member_offset(bt.mstride, mem);
  const int reg = strided_rows(1 << LGZ) * TP;
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  E v[8];
  // all three fields' columns are copied asynchronously into their regions
  // at once (one commit group per field), so the loads of fields 1 and 2 run
  // behind the transform of field 0
  for (int f = 0; f < 3; ++f) {
    const C* in = reinterpret_cast<const C*>(w.at(f));
    E* S = sm + f * reg;
#pragma unroll
    for (int i = 0; i < 8; ++i)
      load_cols_async<R, W>(S + idx(t + i * T), in, (size_t)(t + i * T) * plane + base, X0, ylim);
    cp_async_commit();
  }
  for (int f = 0; f < 3; ++f) {
    E* S = sm + f * reg;
    cp_async_wait(2 - f);   // this thread's copies of field f have landed
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
    __syncthreads();        // every thread holds its inputs before the exchanges overwrite the region
    fft_line_ct<-1, R, LGZ>(v, t, tw, S, idx);
#pragma unroll
    for (int i = 0; i < 8; ++i) S[idx(t + i * T)] = v[i];
  }
  if (!valid) return;  // no barrier follows
  zfwd_epilogue<R, LGZ, W>(sm, reg, idx, t, X0, y, ylim, base, plane, bc, out, tb, g, mode, pruned);
}

// ---------------------------------------------------------------------------
// Pass 5 on a cluster pair of CTAs (FP32, z_cluster = 1).  CTA r of the pair
// holds z-rows [r H, r H + H) (H = nz / 2) of the tile's three fields, half
// the shared memory of k_zfwd_epi, so that two CTAs of different tiles share
// an SM and one's loads and stores run while the other transforms (one
// 16-column tile per SM leaves the SM idle on memory while it transforms, and
// idle on arithmetic while it loads).  The first radix-2 stage of the length-
// nz forward transform (decimation in frequency) pairs row e of CTA 0 with
// row e of CTA 1: y0_e = x_e + x_{e+H} gives the even modes, y1_e =
// (x_e - x_{e+H}) W_nz^e the odd ones; each CTA reads the other's half from
// distributed shared memory, transforms its own with the length-H line
// transform and runs the epilogue for its modes z = 2 k + r.  The tile list,
// columns, pruning and epilogue are those of k_zfwd_epi.
// ---------------------------------------------------------------------------
// Two adjacent columns per thread (CTAs of up to 256 threads).
template <int LGZ>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kSpassThreads, 2)
k_zfwd_cl(Ptr6 w, Ptr6 bc, Ptr6 out, DevTables<float> tb, Geom g, int lgTX, int mode, int pruned,
          const int32_t* __restrict__ tiles, Batch<float> bt) {
  using R = float;
  using C = float2;
  constexpr int W = 2;
  using E = CPair<float>;
  constexpr int LGH = LGZ - 1, H = 1 << LGH, T = H / 8;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  cooperative_groups::cluster_group cluster = cooperative_groups::this_cluster();
  const int r = (int)cluster.block_rank();
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  const unsigned pair = blockIdx.x >> 1;
  int tile = (int)pair, y = blockIdx.y;
  if (pruned) {
    tile = tiles[2 * pair];
    y = tiles[2 * pair + 1];
  }
  const int X0 = tile * TX + W * xp;
  const int ylim = pruned ? tb.xcut[y] : g.nh;
  const bool valid = X0 < ylim;
  const size_t plane = (size_t)g.ny * g.nhp;
  const unsigned mem = pruned ? blockIdx.y : blockIdx.z;
  member_tables(bt, mem, tb);
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0) + member_offset(bt.mstride, mem);
  const int reg = strided_rows(H) * TP;
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  const C* twh = reinterpret_cast<const C*>(tb.twzh);
  // this CTA's rows r H + e of the three fields
  for (int f = 0; f < 3; ++f) {
    const C* in = reinterpret_cast<const C*>(w.at(f));
    E* S = sm + f * reg;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = t + i * T;
      load_cols_async<R, W>(S + idx(e), in, (size_t)(r * H + e) * plane + base, X0, ylim);
    }
  }
  cp_async_commit();
  cp_async_wait(0);
  __syncthreads();
  cluster.sync();   // both halves are in shared memory
  E v[8];
  for (int f = 0; f < 3; ++f) {
    E* S = sm + f * reg;
    const E* P = cluster.map_shared_rank(S, r ^ 1);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = t + i * T;
      const E a = S[idx(e)], b = P[idx(e)];
      if (r == 0) {
        v[i] = cadd(a, b);                      // x_e + x_{e+H}
      } else {
        v[i] = twmul<-1>(csub(b, a), tw[e]);    // (x_e - x_{e+H}) W_nz^e
      }
    }
    cluster.sync();   // both CTAs have read region f before either transform overwrites it
    fft_line_ct<-1, R, LGH>(v, t, twh, S, idx);
#pragma unroll
    for (int i = 0; i < 8; ++i) S[idx(t + i * T)] = v[i];
  }
  // no access to the other CTA's shared memory follows the last cluster barrier
  if (!valid) return;
  zfwd_epilogue<R, LGH, W>(sm, reg, idx, t, X0, y, ylim, base, plane, bc, out, tb, g, mode, pruned, 2, r);
}

// ---------------------------------------------------------------------------
// Pass 5 with its tile loaded by TMA (FP32, 16-column tiles, one column per
// thread, z_tma = 1).  One thread issues the tensor copies of the three
// fields (boxes of 32 floats x min(nz, 256) z-rows), each field completing its
// own mbarrier, so that field 0's transform starts as soon as its rows have
// landed while fields 1 and 2 stream in; with per-thread cp.async copies the
// threads spend about a quarter of a 512^3 tile issuing them.  The regions are
// dense: a row of 16 FP32 columns is one 128-byte line, and every warp access
// of the transforms covers whole rows, so no padding rows are needed against
// bank conflicts.  A box also copies the columns of the tile at or beyond the
// row's limit; those columns are transformed on their own and never stored.
// Every wait is bounded: on a timeout the kernel raises the error flag, waits
// once more (bounded) for its copies and finishes the tile.
// ---------------------------------------------------------------------------

// 2 L threads per block; at most 64 registers, so that shorter lines keep as
// many tiles per SM as their shared memory allows (two of 96 KB at L = 256).
template <int LGZ>
__global__ void __launch_bounds__(2 << LGZ > 1024 ? 1024 : 2 << LGZ,
                                  (2 << LGZ) >= 1024 ? 1 : (1024 / (2 << LGZ) < 4 ? 1024 / (2 << LGZ) : 4))
k_zfwd_tma(const __grid_constant__ CUtensorMap m0, const __grid_constant__ CUtensorMap m1,
           const __grid_constant__ CUtensorMap m2, Ptr6 bc, Ptr6 out, DevTables<float> tb, Geom g, int mode,
           int pruned, const int32_t* __restrict__ tiles, int* err) {
  using R = float;
  using C = float2;
  constexpr int W = 1;
  constexpr int L = 1 << LGZ, T = L / 8, BOX = L < 256 ? L : 256;
  constexpr int TX = 1 << kZTmaLgTX;
  extern __shared__ __align__(128) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + (size_t)3 * L * TX * sizeof(C));
  const int xp = threadIdx.x & (TX - 1), t = threadIdx.x >> kZTmaLgTX;
  int tile = blockIdx.x, y = blockIdx.y;
  if (pruned) {
    tile = tiles[2 * blockIdx.x];
    y = tiles[2 * blockIdx.x + 1];
  }
  const int X0 = tile * TX + xp;
  const int ylim = pruned ? tb.xcut[y] : g.nh;
  const bool valid = X0 < ylim;
  const size_t plane = (size_t)g.ny * g.nhp;
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0);
  const int reg = L * TX;
  const DenseIdxLg idx{kZTmaLgTX, xp};
  if (threadIdx.x == 0) {
    for (int f = 0; f < 3; ++f) mbar_init(&bar[f], 1);
    fence_mbar_init();
    const CUtensorMap* m[3] = {&m0, &m1, &m2};
    for (int f = 0; f < 3; ++f) {
      mbar_arrive_expect_tx(&bar[f], (uint32_t)(L * TX * sizeof(C)));
      for (int h = 0; h < L / BOX; ++h)
        tma_load_3d(sm + f * reg + h * BOX * TX, m[f], tile * 2 * TX, y, h * BOX, &bar[f]);
    }
  }
  __syncthreads();   // the barriers are initialised before anyone waits on them
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  C v[8];
  for (int f = 0; f < 3; ++f) {
    C* S = sm + f * reg;
    if (!mbar_wait(&bar[f], 0)) {   // bounded: record it, and give the copies one more bounded wait
      raise_error(err, GT_ETIMEOUT);
      mbar_wait(&bar[f], 0);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
    __syncthreads();   // every thread holds its inputs before the exchanges overwrite the region
    fft_line_ct<-1, R, LGZ>(v, t, tw, S, idx);
#pragma unroll
    for (int i = 0; i < 8; ++i) S[idx(t + i * T)] = v[i];
  }
  if (!valid) return;   // no barrier follows
  zfwd_epilogue<R, LGZ, W, DenseIdxLg>(sm, reg, idx, t, X0, y, ylim, base, plane, bc, out, tb, g, mode, pruned);
}

// Pass 5 as a persistent kernel (zf_pipe = 1): each block walks the tile list
// (member-major for a batched launch).  The epilogue reads only a thread's own
// shared slots, so as soon as a thread has finished it, the thread copies the
// next tile's three input columns into those same slots (cp.async); the
// barrier before the next tile's first exchange orders them after every
// thread's epilogue.  The next tile's loads thus run behind the current
// tile's epilogue.  Same columns, pruning and results as k_zfwd_epi.
template <typename R, int LGZ>
__global__ void __launch_bounds__(max_threads<R>() / zfwd_cols<R>())
k_zfwd_epi_pf(Ptr6 w, Ptr6 bc, Ptr6 out, DevTables<R> tb0, Geom g, int lgTX, int mode, int pruned,
              const int32_t* __restrict__ tiles, Batch<R> bt, int per_member, int ntx, long long nitems) {
  using C = Cplx<R>;
  constexpr int W = zfwd_cols<R>();
  using E = ColT<R, W>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  constexpr int T = 1 << (LGZ - 3);
  const size_t plane = (size_t)g.ny * g.nhp;
  const int reg = strided_rows(1 << LGZ) * TP;
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb0.twz);
  auto locate = [&](long long item, unsigned& mem, int& y, int& X0, int& ylim, size_t& base) {
    mem = (unsigned)(item / per_member);
    const int ti = (int)(item - (long long)mem * per_member);
    int tile;
    if (pruned) {
      tile = tiles[2 * ti];
      y = tiles[2 * ti + 1];
    } else {
      tile = ti % ntx;
      y = ti / ntx;
    }
    X0 = tile * TX + W * xp;
    ylim = pruned ? tb0.xcut[y] : g.nh;
    base = (size_t)y * g.nhp + (X0 < ylim ? X0 : 0) + member_offset(bt.mstride, mem);
  };
  auto prefetch = [&](long long item) {
    unsigned mem;
    int y, X0, ylim;
    size_t base;
    locate(item, mem, y, X0, ylim, base);
    for (int f = 0; f < 3; ++f) {
      const C* in = reinterpret_cast<const C*>(w.at(f));
      E* S = sm + f * reg;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        load_cols_async<R, W>(S + idx(t + i * T), in, (size_t)(t + i * T) * plane + base, X0, ylim);
      cp_async_commit();
    }
  };
  long long item = blockIdx.x;
  if (item < nitems) {
    prefetch(item);
  } else {
    cp_async_commit(); cp_async_commit(); cp_async_commit();
  }
  for (; item < nitems; item += gridDim.x) {
    unsigned mem;
    int y, X0, ylim;
    size_t base;
    locate(item, mem, y, X0, ylim, base);
    DevTables<R> tb = tb0;
    member_tables(bt, mem, tb);
    E v[8];
    for (int f = 0; f < 3; ++f) {
      E* S = sm + f * reg;
      cp_async_wait(2 - f);   // this thread's copies of field f have landed
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
      __syncthreads();        // every thread holds its inputs (and has left the previous epilogue)
      fft_line_ct<-1, R, LGZ>(v, t, tw, S, idx);
#pragma unroll
      for (int i = 0; i < 8; ++i) S[idx(t + i * T)] = v[i];
    }
    if (X0 < ylim) zfwd_epilogue<R, LGZ, W>(sm, reg, idx, t, X0, y, ylim, base, plane, bc, out, tb, g, mode, pruned);
    if (item + gridDim.x < nitems) {
      prefetch(item + gridDim.x);   // into this thread's own slots, which its epilogue has finished with
    } else {
      cp_async_commit(); cp_async_commit(); cp_async_commit();
    }
  }
  cp_async_wait(0);   // nothing in flight at exit
}


// ---------------------------------------------------------------------------
// Passes 5 and 1 of the RK2 step fused at the stage boundary: the forward z
// transform of the first nonlinear term and its stage-1 epilogue give
// c = emk (b + dt2 N1) (rkstep.f90:30-48), which stays in shared memory
// (regions 0-2, written in place of the transformed N1 at each thread's own
// positions); the inverse z transforms of u = curl c and w = k^2 c for the
// second nonlinear term (nlt.f90:26-40, produ.f90:44-63) follow, with region
// 3 as their scratch.  c is never written to or read back from HBM.  One
// column per thread; the same tiles and pruning as the two separate passes.
// ---------------------------------------------------------------------------
template <typename R, int LGZ>
__global__ void __launch_bounds__(max_threads<R>() / 2 / zcols<R>())
k_zfwd_zinv(Ptr6 w, Ptr6 bc, DevTables<R> tb, Geom g, int lgTX, int pruned, const int32_t* __restrict__ tiles,
            Batch<R> bt) {
  using C = Cplx<R>;
  constexpr int W = zcols<R>();
  using E = ColT<R, W>;
  extern __shared__ __align__(16) unsigned char smraw[];
  E* sm = reinterpret_cast<E*>(smraw);
  const int TX = 1 << lgTX, lgTP = lgTX - (W - 1), TP = 1 << lgTP;
  const int xp = threadIdx.x & (TP - 1), t = threadIdx.x >> lgTP;
  int tile = blockIdx.x, y = blockIdx.y;
  if (pruned) {
    tile = tiles[2 * blockIdx.x];
    y = tiles[2 * blockIdx.x + 1];
  }
  const int X0 = tile * TX + W * xp;
  const int ylim = pruned ? tb.xcut[y] : g.nh;
  const bool valid = X0 < ylim;
  constexpr int T = 1 << (LGZ - 3);
  const size_t plane = (size_t)g.ny * g.nhp;
  const unsigned mem = pruned ? blockIdx.y : blockIdx.z;
  member_tables(bt, mem, tb);
  const size_t base = (size_t)y * g.nhp + (valid ? X0 : 0) + member_offset(bt.mstride, mem);
  const int reg = strided_rows(1 << LGZ) * TP;
  const StridedIdxLg idx{lgTP, xp};
  const C* tw = reinterpret_cast<const C*>(tb.twz);
  E v[8];
  // forward z transforms of N1 (three fields) into regions 0-2
  for (int f = 0; f < 3; ++f) {
    const C* in = reinterpret_cast<const C*>(w.at(f));
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = load_cols<R, W>(in, (size_t)(t + i * T) * plane + base, X0, ylim);
    E* S = sm + f * reg;
    fft_line_ct<-1, R, LGZ>(v, t, tw, S, idx);
#pragma unroll
    for (int i = 0; i < 8; ++i) S[idx(t + i * T)] = v[i];
  }
  // stage-1 epilogue at this thread's own positions: c in place of N1, zero
  // where the separate epilogue would not write
  R kx[W], kxs[W];
#pragma unroll
  for (int c = 0; c < W; ++c) {
    const bool in = X0 + c < ylim;
    kx[c] = in ? tb.fkx[X0 + c] : (R)0;
    kxs[c] = in ? tb.fkxs[X0 + c] : (R)0;
  }
  const R ky = tb.fky[y], kys = tb.fkys[y];
  const C* b0p = reinterpret_cast<const C*>(bc.p[0]);
  const C* b1p = reinterpret_cast<const C*>(bc.p[1]);
  const C* b2p = reinterpret_cast<const C*>(bc.p[2]);
#pragma unroll 2
  for (int i = 0; i < 8; ++i) {
    const int z = t + i * T;
    const int zlim = tb.xcut[(size_t)z * g.ny + y];
    const int wlim = pruned ? zlim : ylim;   // columns the separate epilogue writes
    const size_t o = (size_t)z * plane + base;
    E n0 = sm[idx(z)], n1 = sm[reg + idx(z)], n2 = sm[2 * reg + idx(z)];
    E bb0 = load_cols<R, W>(b0p, o, X0, wlim), bb1 = load_cols<R, W>(b1p, o, X0, wlim),
      bb2 = load_cols<R, W>(b2p, o, X0, wlim);
    const R kz = tb.fkz[z], kzs = tb.fkzs[z];
    const R okz = tb.omega * kz;   // nlt.f90:67-81
#pragma unroll
    for (int c = 0; c < W; ++c) {
      const int X = X0 + c;
      const bool zero_mode = (X == 0) && (y == 0) && (z == 0);
      C s0{0, 0}, s1{0, 0}, s2{0, 0};
      if (X < wlim && !zero_mode) {           // rkstep.f90:44-48: c(0) = 0
        const C b0 = col(bb0, c), b1 = col(bb1, c), b2 = col(bb2, c);
        const C m0 = col(n0, c), m1 = col(n1, c), m2 = col(n2, c);
        const C a0{m0.x - okz * b0.y, m0.y + okz * b0.x};
        const C a1{m1.x - okz * b1.y, m1.y + okz * b1.x};
        const C a2{m2.x - okz * b2.y, m2.y + okz * b2.x};
        const R k2 = (kxs[c] + kys) + kzs;
        const R ik2 = (R)1 / k2;               // produ.f90:83-99
        const R qx = kx[c] * ik2, qy = ky * ik2, qz = kz * ik2;
        C r0{-qy * a2.y + qz * a1.y, qy * a2.x - qz * a1.x};
        C r1{-qz * a0.y + qx * a2.y, qz * a0.x - qx * a2.x};
        C r2{-qx * a1.y + qy * a0.y, qx * a1.x - qy * a0.x};
        if (tb.truncate && X >= zlim) {        // trunc.f90:14-28
          r0 = C{0, 0}; r1 = C{0, 0}; r2 = C{0, 0};
        }
        const R e = tb.emk_by_k2 ? tb.emk[(int)k2] : tb.emk[((size_t)z * g.ny + y) * g.nh + X];
        const R d = tb.dt2;                    // rkstep.f90:30-40
        s0 = C{e * (b0.x + d * r0.x), e * (b0.y + d * r0.y)};
        s1 = C{e * (b1.x + d * r1.x), e * (b1.y + d * r1.y)};
        s2 = C{e * (b2.x + d * r2.x), e * (b2.y + d * r2.y)};
      }
      col(n0, c) = s0;
      col(n1, c) = s1;
      col(n2, c) = s2;
    }
    sm[idx(z)] = n0;
    sm[reg + idx(z)] = n1;
    sm[2 * reg + idx(z)] = n2;
  }
  // inverse z transforms of u = curl c and w = k^2 c from this thread's own
  // positions of c, with region 3 as scratch
  E* S3 = sm + 3 * reg;
#pragma unroll 1
  for (int f = 0; f < 6; ++f) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int z = t + i * T;
      const R kz = tb.fkz[z];
      E q0 = sm[idx(z)], q1 = sm[reg + idx(z)], q2 = sm[2 * reg + idx(z)];
      E r;
#pragma unroll
      for (int c = 0; c < W; ++c) {
        const C p0 = col(q0, c), p1 = col(q1, c), p2 = col(q2, c);
        if (f == 0) {
          col(r, c) = C{-ky * p2.y + kz * p1.y, ky * p2.x - kz * p1.x};
        } else if (f == 1) {
          col(r, c) = C{-kz * p0.y + kx[c] * p2.y, kz * p0.x - kx[c] * p2.x};
        } else if (f == 2) {
          col(r, c) = C{-kx[c] * p1.y + ky * p0.y, kx[c] * p1.x - ky * p0.x};
        } else {
          const R k2 = (kxs[c] + kys) + tb.fkzs[z];
          const C q = f == 3 ? p0 : (f == 4 ? p1 : p2);
          col(r, c) = C{k2 * q.x, k2 * q.y};
        }
      }
      v[i] = r;
    }
    fft_line_ct<+1, R, LGZ>(v, t, tw, S3, idx);
    C* out = reinterpret_cast<C*>(w.at(f));
#pragma unroll
    for (int i = 0; i < 8; ++i) store_cols<R, W>(out, (size_t)(t + i * T) * plane + base, X0, ylim, v[i]);
  }
}

// ---------------------------------------------------------------------------
// Plain x transforms (rows of one field packed in pairs).
// ---------------------------------------------------------------------------
template <typename R, int LGN>
__global__ void __launch_bounds__(max_threads<R>())
k_xc2r(const void* specv, R* __restrict__ real, Geom g, const void* twv, int P) {
  using C = Cplx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int N = 1 << LGN, lgT = LGN - 3, T = 1 << lgT;
  constexpr int LP = N;
  const int p = threadIdx.x >> lgT, t = threadIdx.x & (T - 1);
  const size_t pair = (size_t)blockIdx.x * P + p;
  const C* spec = reinterpret_cast<const C*>(specv);
  const C* X1 = spec + (2 * pair) * g.nhp;
  const C* X2 = spec + (2 * pair + 1) * g.nhp;
  C v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = pack_c2r<R>(X1, X2, t + i * T, N, g.nh);
  fft_line_ct<+1, R, LGN>(v, t, reinterpret_cast<const C*>(twv), sm, SwzIdx{p * LP});
  R* r0 = real + (2 * pair) * (size_t)N;
  R* r1 = real + (2 * pair + 1) * (size_t)N;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    r0[t + i * T] = v[i].x;
    r1[t + i * T] = v[i].y;
  }
}

template <typename R, int LGN>
__global__ void __launch_bounds__(max_threads<R>())
k_xr2c(const R* __restrict__ real, void* specv, Geom g, const void* twv, int P, R shalf) {
  using C = Cplx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  constexpr int N = 1 << LGN, lgT = LGN - 3, T = 1 << lgT;
  constexpr int LP = N;
  const int p = threadIdx.x >> lgT, t = threadIdx.x & (T - 1);
  const size_t pair = (size_t)blockIdx.x * P + p;
  const R* r0 = real + (2 * pair) * (size_t)N;
  const R* r1 = real + (2 * pair + 1) * (size_t)N;
  C v[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = C{r0[t + i * T], r1[t + i * T]};
  const SwzIdx idx{p * LP};
  fft_line_ct<-1, R, LGN>(v, t, reinterpret_cast<const C*>(twv), sm, idx);
#pragma unroll
  for (int i = 0; i < 8; ++i) sm[idx(t + i * T)] = v[i];
  __syncthreads();
  C* spec = reinterpret_cast<C*>(specv);
  const int nh = g.nh;
  for (int n = threadIdx.x; n < P * 2 * nh; n += blockDim.x) {
    const int k = n % nh, rest = n / nh, r = rest & 1, pp = rest >> 1;
    const int o = pp * LP;
    const int kb = (N - k) & (N - 1);
    const C a = sm[o + swz(k)], b = sm[o + swz(kb)];
    const size_t row = 2 * ((size_t)blockIdx.x * P + pp) + r;
    spec[row * g.nhp + k] = split_r2c<R>(a, b, r == 0, shalf);
  }
}

// ---------------------------------------------------------------------------
// Pointwise spectral operators over all modes (output and initial-state
// paths): 0 curl, 1 invcurl, 2 trunc, 3 incompr (with |k.a|^2 partials).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_point(Ptr6 a, DevTables<R> tb, Geom g, int op, double* partial) {
  using C = Cplx<R>;
  __shared__ double red[256];
  double acc = 0.0;
  const size_t rows = (size_t)g.ny * g.nz;
  for (size_t row = blockIdx.y; row < rows; row += gridDim.y) {
    const int y = (int)(row % g.ny), z = (int)(row / g.ny);
    for (int X = blockIdx.x * blockDim.x + threadIdx.x; X < g.nh; X += gridDim.x * blockDim.x) {
      const size_t o = row * g.nhp + X;
      C* p0 = reinterpret_cast<C*>(a.p[0]);
      C* p1 = reinterpret_cast<C*>(a.p[1]);
      C* p2 = reinterpret_cast<C*>(a.p[2]);
      const C ax = p0[o], ay = p1[o], az = p2[o];
      const R kx = tb.fkx[X], ky = tb.fky[y], kz = tb.fkz[z];
      const bool zero_mode = (X == 0) && (y == 0) && (z == 0);
      const R k2 = (tb.fkxs[X] + tb.fkys[y]) + tb.fkzs[z];
      if (op == 0) {  // produ.f90:44-63
        p0[o] = C{-ky * az.y + kz * ay.y, ky * az.x - kz * ay.x};
        p1[o] = C{-kz * ax.y + kx * az.y, kz * ax.x - kx * az.x};
        p2[o] = C{-kx * ay.y + ky * ax.y, kx * ay.x - ky * ax.x};
      } else if (op == 1) {  // produ.f90:79-101
        if (zero_mode) continue;
        const R qx = kx / k2, qy = ky / k2, qz = kz / k2;
        p0[o] = C{-qy * az.y + qz * ay.y, qy * az.x - qz * ay.x};
        p1[o] = C{-qz * ax.y + qx * az.y, qz * ax.x - qx * az.x};
        p2[o] = C{-qx * ay.y + qy * ax.y, qx * ay.x - qy * ax.x};
      } else if (op == 2) {  // trunc.f90:10-28
        if (zero_mode || X >= tb.xcut[(size_t)z * g.ny + y]) {
          p0[o] = C{0, 0}; p1[o] = C{0, 0}; p2[o] = C{0, 0};
        }
      } else {  // trunc.f90:47-63 with the reduction made explicit
        if (zero_mode) continue;
        const C s{kx * ax.x + ky * ay.x + kz * az.x, kx * ax.y + ky * ay.y + kz * az.y};
        acc += (double)s.x * (double)s.x + (double)s.y * (double)s.y;
        p0[o] = C{ax.x - s.x * kx / k2, ax.y - s.y * kx / k2};
        p1[o] = C{ay.x - s.x * ky / k2, ay.y - s.y * ky / k2};
        p2[o] = C{az.x - s.x * kz / k2, az.y - s.y * kz / k2};
      }
    }
  }
  if (op == 3) {
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
  }
}

// ---------------------------------------------------------------------------
// Forcing scatter (forcing_3d3c.f90:45-68, forcing_2d2c.f90:37-41): the host
// drew the increments with the reference RNG; entries are added in order.
// With no repeated mode in a step the adds commute and run one per thread.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_force(Ptr6 b, const ForceEntry* __restrict__ e, int n, int serial, Geom g) {
  using C = Cplx<R>;
  const int first = serial ? 0 : blockIdx.x * blockDim.x + threadIdx.x;
  const int last = serial ? (threadIdx.x == 0 && blockIdx.x == 0 ? n : 0) : first + 1;
  for (int m = first; m < last && m < n; ++m) {
    const ForceEntry en = e[m];
    const size_t o = ((size_t)en.z * g.ny + en.y) * g.nhp + en.x;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (!(en.mask & (1 << c))) continue;
      C* p = reinterpret_cast<C*>(b.at(c));
      if (sizeof(R) == 8) {
        const C v = p[o];
        p[o] = C{(R)((double)v.x + en.inc[2 * c]), (R)((double)v.y + en.inc[2 * c + 1])};
      } else {
        const C v = p[o];
        p[o] = C{v.x + (R)en.inc[2 * c], v.y + (R)en.inc[2 * c + 1]};
      }
    }
  }
}

// Graph-replayable forcing: the entries of every step of a chunk are resident
// ([step][n] in `base`); a device counter selects the step, and k_step_inc
// advances it after the scatter, so one captured graph serves every step.
template <typename R>
__global__ void k_force_indexed(Ptr6 b, const ForceEntry* __restrict__ base, int n,
                                const int* __restrict__ step, Geom g) {
  using C = Cplx<R>;
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const ForceEntry en = base[(size_t)(*step) * n + m];
  const size_t o = ((size_t)en.z * g.ny + en.y) * g.nhp + en.x;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (!(en.mask & (1 << c))) continue;
    C* p = reinterpret_cast<C*>(b.at(c));
    const C v = p[o];
    if (sizeof(R) == 8)
      p[o] = C{(R)((double)v.x + en.inc[2 * c]), (R)((double)v.y + en.inc[2 * c + 1])};
    else
      p[o] = C{v.x + (R)en.inc[2 * c], v.y + (R)en.inc[2 * c + 1]};
  }
}

// Forcing of the members of a batched launch (blockIdx.y = member): member m
// adds its first count[m] entries of step *step; entries [m][nsteps][nmax].
template <typename R>
__global__ void k_force_batch(Ptr6 b, const ForceEntry* __restrict__ base, const int* __restrict__ count,
                              int nmax, int nsteps, const int* __restrict__ step, Geom g, long long mstride) {
  using C = Cplx<R>;
  const unsigned mem = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count[mem]) return;
  const ForceEntry en = base[((size_t)mem * nsteps + *step) * nmax + e];
  const size_t o = ((size_t)en.z * g.ny + en.y) * g.nhp + en.x + member_offset(mstride, mem);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (!(en.mask & (1 << c))) continue;
    C* p = reinterpret_cast<C*>(b.at(c));
    const C v = p[o];
    if (sizeof(R) == 8)
      p[o] = C{(R)((double)v.x + en.inc[2 * c]), (R)((double)v.y + en.inc[2 * c + 1])};
    else
      p[o] = C{v.x + (R)en.inc[2 * c], v.y + (R)en.inc[2 * c + 1]};
  }
}

static __global__ void k_step_inc(int* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1;
}

template <typename R>
__global__ void k_convert(const double2* __restrict__ s64, Cplx<R>* __restrict__ w, size_t n,
                          int to_working) {
  using C = Cplx<R>;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    if (to_working) {
      const double2 v = s64[i];
      w[i] = C{(R)v.x, (R)v.y};
    } else {
      const C v = w[i];
      const_cast<double2*>(s64)[i] = double2{(double)v.x, (double)v.y};
    }
  }
}

// ---------------------------------------------------------------------------
// Diagnostics.  Each warp walks whole (y,z) rows; along a row |k| grows with
// kx, so the shell index is non-decreasing and lanes add to warp-private
// shared bins one lane at a time (fixed order).  Block partials are reduced
// in block order by k_final_sum: the result is bitwise reproducible.
// Scalars: [0..8] glob energy terms, [9..17] enstrophy terms, [18] helicity,
// [19] non-finite count; then E(k) [nbin], E2D(k) [nbin], flux slots [nbin].
// ---------------------------------------------------------------------------
constexpr int kDiagThreads = 256;

template <typename R>
__global__ void __launch_bounds__(kDiagThreads)
k_diag(Ptr6 bb, Ptr6 nn, DevTables<R> tb, Geom g, double nu, double alpnu, double mu, double alpmu,
       int has_flux, double* partials, int nq) {
  using C = Cplx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  double* bins = reinterpret_cast<double*>(smraw);  // [8 warps][3][nbin]
  const int nbin = g.nx / 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < 8 * 3 * nbin; i += blockDim.x) bins[i] = 0.0;
  __syncthreads();
  double s[kDiagScalars];
#pragma unroll
  for (int q = 0; q < kDiagScalars; ++q) s[q] = 0.0;
  double* wb = bins + warp * 3 * nbin;
  const size_t rows = (size_t)g.ny * g.nz;
  const int nwarps = gridDim.x * 8;
  for (size_t row = (size_t)blockIdx.x * 8 + warp; row < rows; row += nwarps) {
    const int y = (int)(row % g.ny), z = (int)(row / g.ny);
    for (int x0 = 0; x0 < g.nh; x0 += 32) {
      const int X = x0 + lane;
      const bool valid = X < g.nh;
      double vsp = 0.0, v2d = 0.0, vfl = 0.0;
      int ib = -1;
      if (valid) {
        const size_t o = row * g.nhp + X;
        const C b0 = reinterpret_cast<const C*>(bb.p[0])[o];
        const C b1 = reinterpret_cast<const C*>(bb.p[1])[o];
        const C b2 = reinterpret_cast<const C*>(bb.p[2])[o];
        const double bx0 = b0.x, by0 = b0.y, bx1 = b1.x, by1 = b1.y, bx2 = b2.x, by2 = b2.y;
        const double kx = tb.fkx[X], ky = tb.fky[y], kz = tb.fkz[z];
        const double k2 = ((double)tb.fkxs[X] + (double)tb.fkys[y]) + (double)tb.fkzs[z];
        const double fac = (X == 0 || X == g.nh - 1) ? 0.5 : 1.0;
        if (!isfinite(bx0) || !isfinite(by0) || !isfinite(bx1) || !isfinite(by1) ||
            !isfinite(bx2) || !isfinite(by2))
          s[19] += 1.0;
        // u = curl b (produ.f90:48-53), w = curl u
        const double ux0 = -ky * by2 + kz * by1, uy0 = ky * bx2 - kz * bx1;
        const double ux1 = -kz * by0 + kx * by2, uy1 = kz * bx0 - kx * bx2;
        const double ux2 = -kx * by1 + ky * by0, uy2 = kx * bx1 - ky * bx0;
        const double wx0 = -ky * uy2 + kz * uy1, wy0 = ky * ux2 - kz * ux1;
        const double wx1 = -kz * uy0 + kx * uy2, wy1 = kz * ux0 - kx * ux2;
        const double wx2 = -kx * uy1 + ky * uy0, wy2 = kx * ux1 - ky * ux0;
        if (k2 > 0.0) {  // diagnostics.f90:132-145
          const double pn = alpnu == 1.0 ? k2 : (alpnu == 0.0 ? 1.0 : pow(k2, alpnu));
          const double pm = alpmu == 1.0 ? k2 : (alpmu == 0.0 ? 1.0 : pow(k2, alpmu));
          const double e0 = fac * (ux0 * ux0 + uy0 * uy0), e1 = fac * (ux1 * ux1 + uy1 * uy1),
                       e2 = fac * (ux2 * ux2 + uy2 * uy2);
          const double z0 = fac * (wx0 * wx0 + wy0 * wy0), z1 = fac * (wx1 * wx1 + wy1 * wy1),
                       z2 = fac * (wx2 * wx2 + wy2 * wy2);
          s[0] += e0; s[1] += e1; s[2] += e2;
          s[3] += 2.0 * nu * e0 * pn; s[4] += 2.0 * nu * e1 * pn; s[5] += 2.0 * nu * e2 * pn;
          s[6] += 2.0 * mu * e0 * pm; s[7] += 2.0 * mu * e1 * pm; s[8] += 2.0 * mu * e2 * pm;
          s[9] += z0; s[10] += z1; s[11] += z2;
          s[12] += 2.0 * nu * z0 * pn; s[13] += 2.0 * nu * z1 * pn; s[14] += 2.0 * nu * z2 * pn;
          s[15] += 2.0 * mu * z0 * pm; s[16] += 2.0 * mu * z1 * pm; s[17] += 2.0 * mu * z2 * pm;
          s[18] += fac * (ux0 * wx0 + uy0 * wy0 + ux1 * wx1 + uy1 * wy1 + ux2 * wx2 + uy2 * wy2);
        }
        const double kk = sqrt(k2);
        ib = (int)kk;
        const double bs = (bx0 * bx0 + by0 * by0) + (bx1 * bx1 + by1 * by1) + (bx2 * bx2 + by2 * by2);
        vsp = kk * kk * fac * bs;                                 // diagnostics.f90:25-26
        if (z == 0) v2d = kk * kk * fac * (bx2 * bx2 + by2 * by2);  // :36-40
        if (has_flux) {                                           // :79-82
          const C n0 = reinterpret_cast<const C*>(nn.p[0])[o];
          const C n1 = reinterpret_cast<const C*>(nn.p[1])[o];
          const C n2 = reinterpret_cast<const C*>(nn.p[2])[o];
          const double sc = (bx0 * n0.x + by0 * n0.y) + (bx1 * n1.x + by1 * n1.y) +
                            (bx2 * n2.x + by2 * n2.y);
          const double f2 = (X == 0 || X == g.nh - 1) ? 1.0 : 2.0;
          vfl = f2 * kk * kk * sc;
        }
      }
      for (int l = 0; l < 32; ++l) {
        if (lane == l && ib >= 0) {
          if (ib + 1 < nbin) {
            wb[ib] += vsp;
            if (z == 0) wb[nbin + ib] += v2d;
          }
          if (has_flux && ib >= 1 && ib < nbin) wb[2 * nbin + ib] += vfl;
        }
        __syncwarp();
      }
    }
  }
  // block reduction of the scalars: warp shuffle tree, then warps in order
  __shared__ double wred[8][kDiagScalars];
#pragma unroll
  for (int q = 0; q < kDiagScalars; ++q) {
    double v = s[q];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) wred[warp][q] = v;
  }
  __syncthreads();
  double* out = partials + (size_t)blockIdx.x * nq;
  if (threadIdx.x < kDiagScalars) {
    double v = 0.0;
    for (int wi = 0; wi < 8; ++wi) v += wred[wi][threadIdx.x];
    out[threadIdx.x] = v;
  }
  for (int i = threadIdx.x; i < 3 * nbin; i += blockDim.x) {
    double v = 0.0;
    for (int wi = 0; wi < 8; ++wi) v += bins[wi * 3 * nbin + i];
    out[kDiagScalars + i] = v;
  }
}

// Kinetic energy per component (diagnostics.f90:126-138 energy terms):
// products in the working precision, accumulation and reduction in FP64.
template <typename R>
__global__ void __launch_bounds__(kDiagThreads)
k_energy(Ptr6 bb, DevTables<R> tb, Geom g, int pruned, double* partials) {
  using C = Cplx<R>;
  constexpr int W = 16 / (int)sizeof(C);   // complex values per 16-byte lane load
  struct alignas(16) U {
    C v[W];
  };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double e0 = 0.0, e1 = 0.0, e2 = 0.0;
  const size_t rows = (size_t)g.ny * g.nz;
  const int nwarps = gridDim.x * (kDiagThreads / 32);
  for (size_t row = (size_t)blockIdx.x * (kDiagThreads / 32) + warp; row < rows; row += nwarps) {
    const int y = (int)(row % g.ny), z = (int)(row / g.ny);
    const R ky = tb.fky[y], kz = tb.fkz[z];
    // pruned: the state is zero outside the kept prefix of the row, whose
    // terms would add exact zeros to the same partial sums
    const int xend = pruned ? tb.xcut[row] : g.nh;
    // a lane's few terms of the row are summed in the working precision, and
    // that sum is added to the FP64 accumulators once per row
    R s0 = 0, s1 = 0, s2 = 0;
#pragma unroll 3
    for (int X0 = W * lane; X0 < xend; X0 += 32 * W) {
      const size_t o = row * g.nhp + X0;   // X0 + W <= nhp: whole 16-byte units of the padded row
      const U u0 = *reinterpret_cast<const U*>(reinterpret_cast<const C*>(bb.p[0]) + o);
      const U u1 = *reinterpret_cast<const U*>(reinterpret_cast<const C*>(bb.p[1]) + o);
      const U u2 = *reinterpret_cast<const U*>(reinterpret_cast<const C*>(bb.p[2]) + o);
#pragma unroll
      for (int c = 0; c < W; ++c) {
        const int X = X0 + c;
        if (X >= xend) break;
        const C b0 = u0.v[c], b1 = u1.v[c], b2 = u2.v[c];
        const R kx = tb.fkx[X];
        const R ux0 = -ky * b2.y + kz * b1.y, uy0 = ky * b2.x - kz * b1.x;
        const R ux1 = -kz * b0.y + kx * b2.y, uy1 = kz * b0.x - kx * b2.x;
        const R ux2 = -kx * b1.y + ky * b0.y, uy2 = kx * b1.x - ky * b0.x;
        const R fac = (X == 0 || X == g.nh - 1) ? (R)0.5 : (R)1;   // k = 0 gives u = 0
        s0 += fac * (ux0 * ux0 + uy0 * uy0);
        s1 += fac * (ux1 * ux1 + uy1 * uy1);
        s2 += fac * (ux2 * ux2 + uy2 * uy2);
      }
    }
    e0 += (double)s0;
    e1 += (double)s1;
    e2 += (double)s2;
  }
  __shared__ double red[kDiagThreads / 32][3];
  for (int off = 16; off > 0; off >>= 1) {
    e0 += __shfl_down_sync(0xffffffffu, e0, off);
    e1 += __shfl_down_sync(0xffffffffu, e1, off);
    e2 += __shfl_down_sync(0xffffffffu, e2, off);
  }
  if (lane == 0) { red[warp][0] = e0; red[warp][1] = e1; red[warp][2] = e2; }
  __syncthreads();
  if (threadIdx.x < 3) {
    double v = 0.0;
    for (int wi = 0; wi < kDiagThreads / 32; ++wi) v += red[wi][threadIdx.x];
    partials[(size_t)blockIdx.x * 3 + threadIdx.x] = v;
  }
}

// result[q] = the sum over b < nblocks of partials[b * nq + q], one block of
// kFinalThreads per quantity: thread t adds the partials b = t, t + kFinalThreads,
// ... in that order, then a fixed tree in shared memory adds the threads' sums,
// so the result does not depend on scheduling.
constexpr int kFinalThreads = 128;
static __global__ void __launch_bounds__(kFinalThreads)
k_final_sum(const double* __restrict__ partials, int nblocks, int nq, double* __restrict__ result) {
  __shared__ double red[kFinalThreads];
  for (int q = blockIdx.x; q < nq; q += gridDim.x) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kFinalThreads) v += partials[(size_t)b * nq + q];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int h = kFinalThreads / 2; h > 0; h >>= 1) {
      if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) result[q] = red[0];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Launch configuration.
// ---------------------------------------------------------------------------
struct SCfg {
  int lgTX, threads, smem, ntiles;
};

static SCfg strided_cfg(int L, int nh, int F, int csize, int maxthreads, int force_tx = 0) {
  const int T = L / 8;
  const int LR = strided_rows(L);   // shared-memory rows of one field (padded)
  if (force_tx > 0) {
    int TX = force_tx;
    while (TX > 1 && (T * TX > maxthreads || F * LR * TX * csize > kSmemForced)) TX >>= 1;
    SCfg c;
    c.lgTX = ilog2i(TX);
    c.threads = T * TX;
    c.smem = F * LR * TX * csize;
    c.ntiles = (nh + TX - 1) / TX;
    return c;
  }
  int TX = 64 / csize;   // 64-byte tile rows: two or more blocks per SM (measured best at 512^3)
  while (TX > 1 && (T * TX > maxthreads || F * LR * TX * csize > kSmemBudget)) TX >>= 1;
  int cap = 1;
  while (cap < nh) cap <<= 1;
  while (T * TX * 2 <= 256 && TX * 2 <= cap && F * LR * TX * 2 * csize <= kSmemBudget &&
         T * TX * 2 <= maxthreads)
    TX <<= 1;
  SCfg c;
  c.lgTX = ilog2i(TX);
  c.threads = T * TX;
  c.smem = F * LR * TX * csize;
  c.ntiles = (nh + TX - 1) / TX;
  return c;
}

// Pairs of rows per block for the x passes.
static int xpass_pairs(const Geom& g, int groups_per_pair, int csize, int maxthreads,
                       int lines_per_pair) {
  const int T = g.nx / 8;
  const int LP = g.nx;
  const long long npairs = (long long)g.ny * g.nz / 2;
  int P = 1;
  while (P * 2 <= npairs && groups_per_pair * T * P * 2 <= maxthreads &&
         groups_per_pair * T * P * 2 <= 256 && lines_per_pair * LP * P * 2 * csize <= kSmemBudget &&
         npairs % (P * 2) == 0)
    P <<= 1;
  return P;
}

// Opt-in dynamic shared memory: the device's per-block maximum minus the
// kernel's static shared memory, set once per (device, precision).
template <typename K>
static cudaError_t allow_smem(K kernel, int optin) {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              optin - (int)fa.sharedSizeBytes);
}

template <typename R>
static int set_smem_attrs() {
  // bit d: device d configured (atomic: handles on other host threads may configure concurrently;
  // setting the attributes twice is harmless)
  static std::atomic<unsigned> done_mask[2] = {{0u}, {0u}};
  const int idx = sizeof(R) == 8 ? 1 : 0;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 32 && (done_mask[idx].load() >> dev) & 1u) return 0;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return (int)e;
  cudaError_t es[8 * 24 + 1];
  int n = 0;
#define GT_ALLOW(LG)                                     \
  es[n++] = allow_smem(k_zinv_curl<R, LG>, optin);       \
  es[n++] = allow_smem(k_zinv_curl_pf<R, LG>, optin);    \
  es[n++] = allow_smem(k_zk2<R, LG>, optin);             \
  es[n++] = allow_smem(k_zinv_curl1<R, LG>, optin);      \
  es[n++] = allow_smem(k_spass<R, 1, LG>, optin);        \
  es[n++] = allow_smem(k_spass<R, -1, LG>, optin);       \
  if (sizeof(R) == 4) {                                  \
    es[n++] = allow_smem(k_spass2<1, LG>, optin);        \
    es[n++] = allow_smem(k_spass2<-1, LG>, optin);       \
    es[n++] = allow_smem(k_spass2_pf<1, LG>, optin);     \
    es[n++] = allow_smem(k_spass2_pf<-1, LG>, optin);    \
    es[n++] = allow_smem(k_zfwd_cl<(LG >= 4 ? LG : 4)>, optin); \
    es[n++] = allow_smem(k_zfwd_tma<(LG >= 4 && LG <= 9 ? LG : 9)>, optin); \
    es[n++] = allow_smem(k_zinv_tma<(LG >= 5 && LG <= 9 ? LG : 9)>, optin); \
    es[n++] = allow_smem(k_zinv_tma<(LG >= 5 && LG <= 9 ? LG : 9), true>, optin); \
  }                                                      \
  es[n++] = allow_smem(k_xcross<R, LG>, optin);          \
  es[n++] = allow_smem(k_xbatch<R, LG>, optin);          \
  es[n++] = allow_smem(k_xbatch<R, LG, true>, optin);    \
  es[n++] = allow_smem(k_zfwd_epi<R, LG>, optin);        \
  es[n++] = allow_smem(k_zfwd_epi_pf<R, LG>, optin);     \
  es[n++] = allow_smem(k_zfwd_zinv<R, LG>, optin);       \
  es[n++] = allow_smem(k_xc2r<R, LG>, optin);            \
  es[n++] = allow_smem(k_xr2c<R, LG>, optin);
  GT_ALLOW(3) GT_ALLOW(4) GT_ALLOW(5) GT_ALLOW(6) GT_ALLOW(7) GT_ALLOW(8) GT_ALLOW(9) GT_ALLOW(10)
#undef GT_ALLOW
  es[n++] = allow_smem(k_diag<R>, optin);
  for (int i = 0; i < n; ++i)
    if (es[i] != cudaSuccess) return (int)es[i];
  if (dev < 32) done_mask[idx].fetch_or(1u << dev);
  return 0;
}

// Blocks of `kernel` resident on the current device at once (one wave); 0
// if the occupancy query fails.
template <typename K>
static int wave_blocks(K kernel, int threads, int smem) {
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess)
    return 0;
  return nsm * per_sm;
}

// Tensor maps of the three z forward pass inputs for TMA boxes of 32 floats
// (16 FP32 complex columns) x 1 row x min(nz, 256) z-planes: dims {2 nhp
// floats, ny, nz}, strides {nhp, ny nhp} complex values.  false when the
// encoder cannot be had or refuses a map (the caller then uses cp.async).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static bool tensor_maps_zcols(const Geom& g, void* const w[], CUtensorMap maps[3], int box_rows = 256) {
  // looked up once (a function-local static: thread-safe initialisation)
  static const EncodeTiledFn enc = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<EncodeTiledFn>(fn);
    return (EncodeTiledFn) nullptr;
  }();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)2 * g.nhp, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
  const cuuint64_t strides[2] = {(cuuint64_t)g.nhp * 8, (cuuint64_t)g.ny * g.nhp * 8};
  const cuuint32_t box[3] = {32, 1, (cuuint32_t)std::min(g.nz, box_rows)};
  const cuuint32_t es[3] = {1, 1, 1};
  for (int f = 0; f < 3; ++f) {
    if (reinterpret_cast<uintptr_t>(w[f]) % 16) return false;
    if (enc(&maps[f], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, w[f], dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return false;
  }
  return true;
}

// SM count of the current device (at least 1).
static int device_sms() {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
    return 1;
  return nsm;
}

// Launches F(LG) for the run-time log2 length lg (3..10).
#define GT_DISPATCH_LG(lg, F)                                                  \
  switch (lg) {                                                                \
    case 3: F(3); break;                                                       \
    case 4: F(4); break;                                                       \
    case 5: F(5); break;                                                       \
    case 6: F(6); break;                                                       \
    case 7: F(7); break;                                                       \
    case 8: F(8); break;                                                       \
    case 9: F(9); break;                                                       \
    case 10: F(10); break;                                                     \
    default: return (int)cudaErrorInvalidValue;                                \
  }

#define GT_HOOK(kind, begin) \
  if (hook) hook(hctx, (kind), (begin))

template <typename R>
static int spass(const Geom& g, void* const* fields, int nf, const void* tw, int axis, int sign,
                 cudaStream_t s, LaunchHook hook, void* hctx, int xlim = -1, int ymask = 0,
                 const int32_t* xcut0 = nullptr, int force_tx = 0, bool pairs = false, int nmem = 1,
                 long long mstride = 0, int prefetch = 0) {
  const int csize = sizeof(Cplx<R>);
  const int L = axis == 1 ? g.ny : g.nz;
  const int lgL = axis == 1 ? g.lny : g.lnz;
  const long long plane = (long long)g.ny * g.nhp;
  const long long ls = axis == 1 ? g.nhp : plane;
  const long long os = axis == 1 ? plane : g.nhp;
  const int outer = axis == 1 ? g.nz : g.ny;
  SCfg c = strided_cfg(L, g.nh, 1, csize, kSpassThreads, force_tx);
  if (xlim < 0) xlim = g.nh;
  const int TX = 1 << c.lgTX;
  Ptr6 f{};
  for (int i = 0; i < nf; ++i) f.p[i] = fields[i];
  const int ntx = (xlim + TX - 1) / TX;
  const int kind = sign > 0 ? kKYPass : kKYFwd;
  if (pairs) {
    // FP32, two columns per thread: the tile is chosen for 2 x kSpassThreads
    // threads of one column each, then halved
    SCfg c2 = strided_cfg(L, g.nh, 1, csize, 2 * kSpassThreads, force_tx);
    if (c2.lgTX >= 1) {
      const int TX2 = 1 << c2.lgTX;
      const int ntx2 = (xlim + TX2 - 1) / TX2;
      if (prefetch) {
        // persistent, double-buffered: as many blocks as fit on the device at once
        const int nsm = device_sms();   // the current device's, every launch
        const long long nitems = (long long)ntx2 * outer * nf * nmem;
        const int threads = c2.threads / 2, smem = 2 * c2.smem;
        GT_HOOK(kind, true);
#define GT_L(LG)                                                                                          \
  {                                                                                                       \
    auto kern = sign > 0 ? k_spass2_pf<1, LG> : k_spass2_pf<-1, LG>;                                      \
    int per_sm = 0;                                                                                       \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess ||    \
        per_sm < 1)                                                                                      \
      per_sm = 1;                                                                                         \
    const unsigned blocks = (unsigned)std::min<long long>(nitems, (long long)per_sm * nsm);              \
    kern<<<blocks, threads, smem, s>>>(f, g, tw, ls, os, c2.lgTX - 1, xlim, ymask, xcut0, nf, mstride,   \
                                       ntx2, outer, nitems);                                              \
  }
        GT_DISPATCH_LG(lgL, GT_L)
#undef GT_L
        GT_HOOK(kind, false);
        return (int)cudaGetLastError();
      }
      dim3 grid2(ntx2, outer, nf * nmem);
      GT_HOOK(kind, true);
#define GT_L(LG)                                                                                      \
  if (sign > 0)                                                                                       \
    k_spass2<1, LG><<<grid2, c2.threads / 2, c2.smem, s>>>(f, g, tw, ls, os, c2.lgTX - 1, xlim, ymask, xcut0, \
                                                            nf, mstride);                                  \
  else                                                                                                \
    k_spass2<-1, LG><<<grid2, c2.threads / 2, c2.smem, s>>>(f, g, tw, ls, os, c2.lgTX - 1, xlim, ymask, xcut0, \
                                                             nf, mstride);
      GT_DISPATCH_LG(lgL, GT_L)
#undef GT_L
      GT_HOOK(kind, false);
      return (int)cudaGetLastError();
    }
  }
  dim3 grid(ntx, outer, nf * nmem);
  GT_HOOK(kind, true);
#define GT_L(LG)                                                                                  \
  if (sign > 0)                                                                                   \
    k_spass<R, 1, LG><<<grid, c.threads, c.smem, s>>>(f, g, tw, ls, os, c.lgTX, xlim, ymask, xcut0, nf, mstride); \
  else                                                                                            \
    k_spass<R, -1, LG><<<grid, c.threads, c.smem, s>>>(f, g, tw, ls, os, c.lgTX, xlim, ymask, xcut0, nf, mstride);
  GT_DISPATCH_LG(lgL, GT_L)
#undef GT_L
  GT_HOOK(kind, false);
  return (int)cudaGetLastError();
}

template <typename R>
// The passes of one nonlinear term; `phases` selects pass 1 (bit 0), passes
// 2-4 (bit 1) and pass 5 (bit 2), so that the RK2 step can run the stage
// boundary as one fused kernel in between.
static int nlt_phases(const Geom& g, const DevTables<R>& tb, void* const a[3], void* const bcor[3],
                      void* const out[3], void* const w[6], int mode, int pruned, const PassTuning* pm,
                      int* err, void* stream, LaunchHook hook, void* hctx, int phases,
                      const Batch<R>* bt = nullptr) {
  int rc = set_smem_attrs<R>();
  if (rc) return rc;
  // a batched launch covers nm members (a spare grid axis), their fields mstride apart
  const Batch<R> bb = bt ? *bt : Batch<R>{};
  const unsigned nm = bb.nmem > 0 ? (unsigned)bb.nmem : 1u;
  const long long mstride = bb.nmem > 0 ? bb.mstride : 0;
  cudaStream_t s = (cudaStream_t)stream;
  const int csize = sizeof(Cplx<R>);
  // z tiles: 16 columns (128-byte row segments, one block of three 512-row
  // fields per SM) for FP32 z columns of 256 points or more, where they
  // measured faster (z forward pass 0.465 -> 0.437 ms at 512^3); else the
  // default width of strided_cfg
  const int ztx = pm && pm->z_tx ? pm->z_tx : (sizeof(R) == 4 && g.lnz >= 8 ? 16 : 0);
  // pass 1's tile shape (three fields per tile)
  const SCfg c1 = strided_cfg(g.nz, g.nh, 3, csize, max_threads<R>(), ztx);
  // overlap: pass 1's k^2 half and pass 2 on the w fields run on a second stream
  // (only where the k^2 half fits its one-region kernel)
  const bool ovl = (phases & 3) == 3 && pm && pm->overlap && pm->stream2 && pm->ev_fork && pm->ev_join &&
                   pm->z_split != 2 && pm->z_split != 3 && c1.threads / zcols<R>() <= kSpassThreads;
  cudaStream_t s2 = ovl ? (cudaStream_t)pm->stream2 : s;
  if (ovl) {
    if ((rc = (int)cudaEventRecord((cudaEvent_t)pm->ev_fork, s))) return rc;
    if ((rc = (int)cudaStreamWaitEvent(s2, (cudaEvent_t)pm->ev_fork, 0))) return rc;
  }
  // pass 1
  if (phases & 1) {
    const SCfg c = c1;
    if (c.lgTX < zcols<R>() - 1) return (int)cudaErrorInvalidConfiguration;   // a column pair per thread
    if (c.lgTX < 0 || c.lgTX > 10) return (int)cudaErrorInvalidConfiguration;   // no tile list
    Ptr6 pa{}, pw{};
    for (int i = 0; i < 3; ++i) pa.p[i] = a[i];
    for (int i = 0; i < 6; ++i) pw.p[i] = w[i];
    const dim3 grid = pruned ? dim3(tb.nztl[c.lgTX], nm) : dim3(c.ntiles, g.ny, nm);
    GT_HOOK(kKZinvCurl, true);
    const bool fits = c.threads / zcols<R>() <= kSpassThreads;
    const int split = (ovl || (pm && pm->z_split == 1)) && fits ? 1 : 0;
    if (ovl && !split) return (int)cudaErrorInvalidConfiguration;
    CUtensorMap amaps[3];
    const bool zitma = sizeof(R) == 4 && pruned && pm && (pm->z_tma & 2) && nm == 1 && !split && !ovl &&
                       pm->z_split == 0 && g.lnz >= 5 && g.lnz <= 9 && tensor_maps_zcols(g, a, amaps, kZBoxRows);
    if (zitma) {
      const int lgt = kZTmaLgTX;
      const int threads = (1 << (lgt - 1)) * (g.nz / 8);
      const int smem = 3 * g.nz * (1 << lgt) * csize + 6 * (int)sizeof(uint64_t);
      const auto& tbf = reinterpret_cast<const DevTables<float>&>(tb);
      // tensor stores of the six outputs (bit 4): boxes of 16 columns x min(nz, 256) rows
      ZOutMaps om{};
      const bool zist = (pm->z_tma & 4) && tensor_maps_zcols(g, w, om.m, 256) &&
                        tensor_maps_zcols(g, w + 3, om.m + 3, 256);
#define GT_L(LG)                                                                                          \
  if (zist)                                                                                               \
    k_zinv_tma<(LG >= 5 && LG <= 9 ? LG : 9), true><<<dim3(tb.nztl[lgt]), threads, smem, s>>>(              \
        amaps[0], amaps[1], amaps[2], om, pw, tbf, g, tb.ztl[lgt], tb.ztlzc[lgt], err);                     \
  else                                                                                                    \
    k_zinv_tma<(LG >= 5 && LG <= 9 ? LG : 9)><<<dim3(tb.nztl[lgt]), threads, smem, s>>>(                    \
        amaps[0], amaps[1], amaps[2], om, pw, tbf, g, tb.ztl[lgt], tb.ztlzc[lgt], err);
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    } else if (pm && pm->z_split == 3 && !ovl) {
      // persistent, software-pipelined: as many blocks as fit on the device at once
      const int nsm = device_sms();   // the current device's, every launch
      const int per_member = pruned ? tb.nztl[c.lgTX] : c.ntiles * g.ny;
      const long long nitems = (long long)per_member * nm;
      const int threads = c.threads / zcols<R>();
#define GT_L(LG)                                                                                         \
  {                                                                                                      \
    int per_sm = 0;                                                                                      \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zinv_curl_pf<R, LG>, threads, c.smem) != \
            cudaSuccess ||                                                                               \
        per_sm < 1)                                                                                      \
      per_sm = 1;                                                                                        \
    const unsigned blocks = (unsigned)std::min<long long>(nitems, (long long)per_sm * nsm);             \
    k_zinv_curl_pf<R, LG><<<blocks, threads, c.smem, s>>>(pa, pw, tb, g, c.lgTX, pruned, tb.ztl[c.lgTX],   \
                                                          per_member, c.ntiles, nitems, mstride);       \
  }
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    } else if (pm && pm->z_split == 2 && fits) {
      // one shared region, the input columns read again per output line
#define GT_L(LG)                                                                                   \
  k_zinv_curl1<R, LG><<<grid, c.threads / zcols<R>(), c.smem / 3, s>>>(pa, pw, tb, g, c.lgTX, pruned, \
                                                                       tb.ztl[c.lgTX], mstride);
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    } else {
#define GT_L(LG)                                                                                   \
  k_zinv_curl<R, LG><<<grid, c.threads / zcols<R>(), c.smem, s>>>(pa, pw, tb, g, c.lgTX, pruned,    \
                                                                  tb.ztl[c.lgTX], split ? 0 : 1, mstride);
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    }
    if (split && !(rc = (int)cudaGetLastError())) {
      // w = k^2 a: one field per block, one shared region (a third of the smem)
      const dim3 grid2 = pruned ? dim3(tb.nztl[c.lgTX], 3, nm) : dim3(c.ntiles, 3, g.ny * nm);
      const int smem1 = c.smem / 3;
#define GT_L(LG) \
  k_zk2<R, LG><<<grid2, c.threads / zcols<R>(), smem1, s2>>>(pa, pw, tb, g, c.lgTX, pruned, tb.ztl[c.lgTX], mstride);
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    }
    GT_HOOK(kKZinvCurl, false);
    if ((rc = (int)cudaGetLastError())) return rc;
  }
  const int xlim = pruned ? tb.xa : g.nh;
  // y passes: 32-byte tile rows for FP32 by default (measured best at 512^3)
  // FP32 y passes with two columns per thread unless switched off; tile
  // columns: 8 with column pairs, 4 without (measured best at 512^3)
  const bool ypairs = sizeof(R) == 4 && (!pm || pm->y_pairs);
  const int ytx = pm && pm->y_tx ? pm->y_tx : (sizeof(R) == 4 ? (ypairs ? 8 : 4) : 0);
  const R shalf = (R)(0.5 / ((double)g.nx * g.ny * g.nz));
  // passes 2-4 (the y and x passes; gs and ws are the grid and work fields)
  const int ypf = pm ? pm->y_prefetch : 1;
  // pass 2 on stream ms (with overlap: u on ms, w on the second stream, joined before pass 3)
  auto pass2 = [&](const Geom& gs, void* const* ws, cudaStream_t ms) -> int {
    int rc2 = 0;
    if ((rc2 = spass<R>(gs, ws, ovl ? 3 : 6, tb.twy, 1, +1, ms, hook, hctx, xlim, pruned ? 1 : 0, tb.xcut, ytx,
                        ypairs, (int)nm, mstride, ypf >= 1 ? 1 : 0)))
      return rc2;
    if (ovl) {
      if ((rc2 = spass<R>(gs, ws + 3, 3, tb.twy, 1, +1, s2, hook, hctx, xlim, pruned ? 1 : 0, tb.xcut, ytx,
                          ypairs, (int)nm, mstride, ypf >= 1 ? 1 : 0)))
        return rc2;
      if ((rc2 = (int)cudaEventRecord((cudaEvent_t)pm->ev_join, s2))) return rc2;
      if ((rc2 = (int)cudaStreamWaitEvent(ms, (cudaEvent_t)pm->ev_join, 0))) return rc2;
    }
    return 0;
  };
  // passes 3 and 4 on stream ms
  auto pass34 = [&](const Geom& gs, void* const* ws, cudaStream_t ms) -> int {
    int rc2 = 0;
    // pass 3
    if (!pm || pm->x_fused) {
      // one group of nx/8 threads per row pair; as many groups per block as
      // fit in xfused_threads and divide the number of row pairs
      const int T = gs.nx / 8;
      const long long npairs = (long long)gs.ny * gs.nz / 2;
      int P = 1;
      while (P * 2 * T <= xfused_threads<R>() && npairs % (P * 2) == 0) P <<= 1;
      if (P * T > xfused_threads<R>() || npairs % P != 0) return (int)cudaErrorInvalidConfiguration;
      const int smem = P * gs.nx * csize;
      Ptr6 pw{};
      for (int i = 0; i < 6; ++i) pw.p[i] = ws[i];
      GT_HOOK(kKXCross, true);
      if (!pm || pm->x_fused == 2) {
#define GT_L(LG) \
  k_xbatch<R, LG><<<dim3((unsigned)(npairs / P), nm), P * T, 3 * smem, ms>>>(pw, gs, tb.twx, shalf, xlim, mstride);
        GT_DISPATCH_LG(gs.lnx, GT_L)
#undef GT_L
      } else if (pm->x_fused == 3) {
        // three planes and the parking region (N complex + N real per group)
        const int psmem = 3 * smem + smem + smem / 2;
#define GT_L(LG) \
  k_xbatch<R, LG, true><<<dim3((unsigned)(npairs / P), nm), P * T, psmem, ms>>>(pw, gs, tb.twx, shalf, xlim, mstride);
        GT_DISPATCH_LG(gs.lnx, GT_L)
#undef GT_L
      } else {
#define GT_L(LG) \
  k_xfused<R, LG><<<dim3((unsigned)(npairs / P), nm), P * T, smem, ms>>>(pw, gs, tb.twx, shalf, xlim, mstride);
        GT_DISPATCH_LG(gs.lnx, GT_L)
#undef GT_L
      }
      GT_HOOK(kKXCross, false);
      if ((rc2 = (int)cudaGetLastError())) return rc2;
    } else {
      const int P = xpass_pairs(gs, 3, csize, max_threads<R>(), 6);
      const int threads = 3 * P * (gs.nx / 8);
      if (threads > (gs.lnx >= 10 ? 384 : 192)) return (int)cudaErrorInvalidConfiguration;
      const int smem = 6 * P * gs.nx * csize;
      const long long nblocks = (long long)gs.ny * gs.nz / 2 / P;
      Ptr6 pw{};
      for (int i = 0; i < 6; ++i) pw.p[i] = ws[i];
      GT_HOOK(kKXCross, true);
#define GT_L(LG) \
  k_xcross<R, LG><<<dim3((unsigned)nblocks, nm), threads, smem, ms>>>(pw, gs, tb.twx, P, shalf, xlim, mstride);
      GT_DISPATCH_LG(gs.lnx, GT_L)
#undef GT_L
      GT_HOOK(kKXCross, false);
      if ((rc2 = (int)cudaGetLastError())) return rc2;
    }
    // pass 4
    return spass<R>(gs, ws, 3, tb.twy, 1, -1, ms, hook, hctx, xlim, pruned ? 2 : 0, tb.xcut, ytx, ypairs,
                    (int)nm, mstride, ypf >= 2 ? 1 : 0);
  };
  // passes 2-4 over the whole grid, or (slab_pipe) over two halves of the
  // z-planes on two streams, the second half's y inverse transform after the
  // first half's, so that one half's x pass runs beside the other half's y
  // passes
  auto middle = [&](const Geom& gs, void* const* ws) -> int {
    const bool sp = pm && pm->slab_pipe && !ovl && pm->stream2 && pm->ev_fork && pm->ev_join &&
                    pm->ev_mid && (gs.nz % 2) == 0 && gs.nz >= 2;
    if (!sp) {
      int rc2 = pass2(gs, ws, s);
      return rc2 ? rc2 : pass34(gs, ws, s);
    }
    cudaStream_t t2 = (cudaStream_t)pm->stream2;
    Geom gh = gs;
    gh.nz = gs.nz / 2;
    const size_t half = (size_t)gh.nz * gs.ny * gs.nhp * (size_t)csize;
    void* wb[6];
    for (int i = 0; i < 6; ++i) wb[i] = static_cast<char*>(ws[i]) + half;
    int rc2;
    if ((rc2 = (int)cudaEventRecord((cudaEvent_t)pm->ev_fork, s))) return rc2;
    if ((rc2 = pass2(gh, ws, s))) return rc2;
    if ((rc2 = (int)cudaEventRecord((cudaEvent_t)pm->ev_mid, s))) return rc2;
    if ((rc2 = (int)cudaStreamWaitEvent(t2, (cudaEvent_t)pm->ev_mid, 0))) return rc2;
    if ((rc2 = pass2(gh, wb, t2))) return rc2;
    if ((rc2 = pass34(gh, wb, t2))) return rc2;
    if ((rc2 = pass34(gh, ws, s))) return rc2;
    if ((rc2 = (int)cudaEventRecord((cudaEvent_t)pm->ev_join, t2))) return rc2;
    return (int)cudaStreamWaitEvent(s, (cudaEvent_t)pm->ev_join, 0);
  };
  if ((phases & 2) && (rc = middle(g, w))) return rc;
  // pass 5
  if (phases & 4) {
    SCfg c = strided_cfg(g.nz, g.nh, 3, csize, max_threads<R>(), ztx);
    if (c.lgTX < zfwd_cols<R>() - 1) return (int)cudaErrorInvalidConfiguration;
    if (c.lgTX < 0 || c.lgTX > 10) return (int)cudaErrorInvalidConfiguration;
    Ptr6 pw{}, pb{}, po{};
    for (int i = 0; i < 3; ++i) {
      pw.p[i] = w[i];
      pb.p[i] = bcor[i];
      po.p[i] = out[i];
    }
    const dim3 grid = pruned ? dim3(tb.nztl[c.lgTX], nm) : dim3(c.ntiles, g.ny, nm);
    GT_HOOK(kKZFwdEpi, true);
    // cluster pairs (z_cluster; the default for FP32 z columns of 1024 points
    // or more, where the one-CTA tiles are 8 columns wide: 4.68 -> 4.31 ms at
    // 1024^3; at 512^3 the 16-column one-CTA tiles are faster, 0.43 against
    // 0.47 ms): tiles of up to 16 columns whose CTAs ((tile / 2) column pairs
    // x nz / 16 threads) fit kSpassThreads
    const int lgcl = std::min(4, 13 - g.lnz);
    CUtensorMap zmaps[3];
    const bool ztma = sizeof(R) == 4 && pm && (pm->z_tma & 1) && nm == 1 && g.lnz >= 4 && g.lnz <= 9 &&
                      !pm->zf_pipe && tensor_maps_zcols(g, w, zmaps);
    if (ztma) {
      // TMA-loaded tiles of 16 columns, one column per thread
      const int threads = (1 << kZTmaLgTX) * (g.nz / 8);
      const int smem = 3 * g.nz * (1 << kZTmaLgTX) * csize + 3 * (int)sizeof(uint64_t);
      const int ntx = (g.nh + (1 << kZTmaLgTX) - 1) >> kZTmaLgTX;
      const dim3 gridt = pruned ? dim3(tb.nztl[kZTmaLgTX]) : dim3(ntx, g.ny);
      const auto& tbf = reinterpret_cast<const DevTables<float>&>(tb);
#define GT_L(LG)                                                                                          \
  k_zfwd_tma<(LG >= 4 && LG <= 9 ? LG : 9)><<<gridt, threads, smem, s>>>(zmaps[0], zmaps[1], zmaps[2], pb, po, \
                                                                         tbf, g, mode, pruned,            \
                                                                         tb.ztl[kZTmaLgTX], err);
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    } else if (sizeof(R) == 4 && pm && pm->z_cluster && !pm->zf_pipe && g.lnz >= 4 && lgcl >= 1) {
      const int TPc = 1 << (lgcl - 1), Hc = g.nz / 2;
      const int threads = TPc * (Hc / 8);
      const int smem = 3 * strided_rows(Hc) * TPc * 2 * csize;
      const int ntx = (g.nh + (1 << lgcl) - 1) >> lgcl;
      const dim3 gridc = pruned ? dim3(2 * tb.nztl[lgcl], nm) : dim3(2 * ntx, g.ny, nm);
      const auto& tbf = reinterpret_cast<const DevTables<float>&>(tb);
      const auto& btf = reinterpret_cast<const Batch<float>&>(bb);
#define GT_L(LG)                                                                                         \
  k_zfwd_cl<(LG >= 4 ? LG : 4)><<<gridc, threads, smem, s>>>(pw, pb, po, tbf, g, lgcl, mode, pruned,     \
                                                             tb.ztl[lgcl], btf);
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    } else if (pm && pm->zf_pipe) {
      // persistent: as many blocks as fit on the device at once
      const int nsm = device_sms();   // the current device's, every launch
      const int per_member = pruned ? tb.nztl[c.lgTX] : c.ntiles * g.ny;
      const long long nitems = (long long)per_member * nm;
      const int threads = c.threads / zfwd_cols<R>();
#define GT_L(LG)                                                                                          \
  {                                                                                                       \
    int per_sm = 0;                                                                                       \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zfwd_epi_pf<R, LG>, threads, c.smem) !=  \
            cudaSuccess ||                                                                                \
        per_sm < 1)                                                                                       \
      per_sm = 1;                                                                                         \
    const unsigned blocks = (unsigned)std::min<long long>(nitems, (long long)per_sm * nsm);              \
    k_zfwd_epi_pf<R, LG><<<blocks, threads, c.smem, s>>>(pw, pb, po, tb, g, c.lgTX, mode, pruned,        \
                                                         tb.ztl[c.lgTX], bb, per_member, c.ntiles, nitems); \
  }
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    } else {
#define GT_L(LG)                                                                                   \
  k_zfwd_epi<R, LG><<<grid, c.threads / zfwd_cols<R>(), c.smem, s>>>(pw, pb, po, tb, g, c.lgTX, mode, \
                                                                 pruned, tb.ztl[c.lgTX], bb);
      GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    }
    GT_HOOK(kKZFwdEpi, false);
    if ((rc = (int)cudaGetLastError())) return rc;
  }
  return 0;
}

template <typename R>
int launch_nlt(const Geom& g, const DevTables<R>& tb, void* const a[3], void* const bcor[3],
               void* const out[3], void* const w[6], int mode, int pruned, const PassTuning* pm,
               int* err, void* stream, LaunchHook hook, void* hctx) {
  return nlt_phases<R>(g, tb, a, bcor, out, w, mode, pruned, pm, err, stream, hook, hctx, 7);
}

// Both nonlinear terms of one RK2 step (main.f90:124-146): b -> c -> b.  With
// fuse_stage the first term's pass 5 and the second term's pass 1 run as the
// fused k_zfwd_zinv (c stays on chip; four shared regions per tile, which
// lowers occupancy: slower than the two passes at 512^3, 1.19 against 1.05 ms);
// otherwise c goes through HBM.
template <typename R>
int launch_rk2_nlts(const Geom& g, const DevTables<R>& tb, void* const b[3], void* const c[3],
                    void* const w[6], int pruned, const PassTuning* pm, int* err, void* stream,
                    LaunchHook hook, void* hctx, const Batch<R>* bt) {
  const bool fuse = pm && pm->fuse_stage;
  if (!fuse) {
    int rc = nlt_phases<R>(g, tb, b, b, c, w, kStage1, pruned, pm, err, stream, hook, hctx, 7, bt);
    if (rc) return rc;
    return nlt_phases<R>(g, tb, c, b, b, w, kStage2, pruned, pm, err, stream, hook, hctx, 7, bt);
  }
  const Batch<R> bb = bt ? *bt : Batch<R>{};
  const unsigned nm = bb.nmem > 0 ? (unsigned)bb.nmem : 1u;
  int rc = nlt_phases<R>(g, tb, b, b, c, w, kStage1, pruned, pm, err, stream, hook, hctx, 1 | 2, bt);
  if (rc) return rc;
  {
    const int csize = sizeof(Cplx<R>);
    cudaStream_t s = (cudaStream_t)stream;
    // four regions per tile; 8 columns (FP32, as column pairs) / 2 (FP64) by default
    SCfg cf = strided_cfg(g.nz, g.nh, 4, csize, max_threads<R>() / 2 * zcols<R>(),
                          pm && pm->z_tx ? pm->z_tx : (sizeof(R) == 4 ? 8 : 2));
    if (cf.lgTX < zcols<R>() - 1 || cf.lgTX > 10) return (int)cudaErrorInvalidConfiguration;
    Ptr6 pw{}, pb{};
    for (int i = 0; i < 6; ++i) pw.p[i] = w[i];
    for (int i = 0; i < 3; ++i) pb.p[i] = b[i];
    const dim3 grid = pruned ? dim3(tb.nztl[cf.lgTX], nm) : dim3(cf.ntiles, g.ny, nm);
    GT_HOOK(kKZFwdZinv, true);
#define GT_L(LG)                                                                                  \
  k_zfwd_zinv<R, LG><<<grid, cf.threads / zcols<R>(), cf.smem, s>>>(pw, pb, tb, g, cf.lgTX, pruned, \
                                                                   tb.ztl[cf.lgTX], bb);
    GT_DISPATCH_LG(g.lnz, GT_L)
#undef GT_L
    GT_HOOK(kKZFwdZinv, false);
    if ((rc = (int)cudaGetLastError())) return rc;
  }
  return nlt_phases<R>(g, tb, c, b, b, w, kStage2, pruned, pm, err, stream, hook, hctx, 2 | 4, bt);
}

template <typename R>
int launch_force(const Geom& g, void* const b[3], const ForceEntry* entries, int n, int serial,
                 void* stream, LaunchHook hook, void* hctx) {
  if (n <= 0) return 0;
  Ptr6 pb{};
  for (int i = 0; i < 3; ++i) pb.p[i] = b[i];
  const int threads = 128;
  const int blocks = serial ? 1 : (n + threads - 1) / threads;
  GT_HOOK(kKForce, true);
  k_force<R><<<blocks, threads, 0, (cudaStream_t)stream>>>(pb, entries, n, serial, g);
  GT_HOOK(kKForce, false);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_force_indexed(const Geom& g, void* const b[3], const ForceEntry* base, int n,
                         const int* step, void* stream, LaunchHook hook, void* hctx) {
  Ptr6 pb{};
  for (int i = 0; i < 3; ++i) pb.p[i] = b[i];
  GT_HOOK(kKForce, true);
  if (n > 0)
    k_force_indexed<R><<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(pb, base, n, step, g);
  k_step_inc<<<1, 32, 0, (cudaStream_t)stream>>>(const_cast<int*>(step));
  GT_HOOK(kKForce, false);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_force_batch(const Geom& g, void* const b[3], const Batch<R>& bt, const ForceEntry* base,
                       const int* count, int nmax, int nsteps, const int* step, void* stream,
                       LaunchHook hook, void* hctx) {
  Ptr6 pb{};
  for (int i = 0; i < 3; ++i) pb.p[i] = b[i];
  GT_HOOK(kKForce, true);
  if (nmax > 0 && bt.nmem > 0)
    k_force_batch<R><<<dim3((nmax + 127) / 128, bt.nmem), 128, 0, (cudaStream_t)stream>>>(
        pb, base, count, nmax, nsteps, step, g, bt.mstride);
  k_step_inc<<<1, 32, 0, (cudaStream_t)stream>>>(const_cast<int*>(step));
  GT_HOOK(kKForce, false);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_convert(const Geom& g, const void* src, void* dst, int to_working, void* stream,
                   LaunchHook hook, void* hctx) {
  const size_t n = g.field_elems();
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((n + threads - 1) / threads, 152 * 16);
  GT_HOOK(kKConvert, true);
  if (to_working)
    k_convert<R><<<blocks, threads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const double2*>(src), reinterpret_cast<Cplx<R>*>(dst), n, 1);
  else
    k_convert<R><<<blocks, threads, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const double2*>(dst), reinterpret_cast<Cplx<R>*>(const_cast<void*>(src)),
        n, 0);
  GT_HOOK(kKConvert, false);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_fft_inv(const Geom& g, const DevTables<R>& tb, void* spec, void* real_out,
                   void* const w[6], void* stream, LaunchHook hook, void* hctx) {
  int rc = set_smem_attrs<R>();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  (void)w;
  void* f[1] = {spec};
  if ((rc = spass<R>(g, f, 1, tb.twz, 2, +1, s, hook, hctx))) return rc;
  if ((rc = spass<R>(g, f, 1, tb.twy, 1, +1, s, hook, hctx))) return rc;
  const int csize = sizeof(Cplx<R>);
  const int P = xpass_pairs(g, 1, csize, max_threads<R>(), 1);
  const int LP = g.nx;
  const long long nblocks = (long long)g.ny * g.nz / 2 / P;
  GT_HOOK(kKFft1, true);
#define GT_L(LG)                                                                    \
  k_xc2r<R, LG><<<(unsigned)nblocks, P * (g.nx / 8), P * LP * csize, s>>>(            \
      spec, reinterpret_cast<R*>(real_out), g, tb.twx, P);
  GT_DISPATCH_LG(g.lnx, GT_L)
#undef GT_L
  GT_HOOK(kKFft1, false);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_fft_dir(const Geom& g, const DevTables<R>& tb, const void* real_in, void* spec_out,
                   void* const w[6], void* stream, LaunchHook hook, void* hctx) {
  int rc = set_smem_attrs<R>();
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  (void)w;
  const int csize = sizeof(Cplx<R>);
  const int P = xpass_pairs(g, 1, csize, max_threads<R>(), 1);
  const int LP = g.nx;
  const long long nblocks = (long long)g.ny * g.nz / 2 / P;
  const R shalf = (R)(0.5 / ((double)g.nx * g.ny * g.nz));
  GT_HOOK(kKFft1, true);
#define GT_L(LG)                                                                    \
  k_xr2c<R, LG><<<(unsigned)nblocks, P * (g.nx / 8), P * LP * csize, s>>>(            \
      reinterpret_cast<const R*>(real_in), spec_out, g, tb.twx, P, shalf);
  GT_DISPATCH_LG(g.lnx, GT_L)
#undef GT_L
  GT_HOOK(kKFft1, false);
  if ((rc = (int)cudaGetLastError())) return rc;
  void* f[1] = {spec_out};
  if ((rc = spass<R>(g, f, 1, tb.twy, 1, -1, s, hook, hctx))) return rc;
  return spass<R>(g, f, 1, tb.twz, 2, -1, s, hook, hctx);
}

template <typename R>
int launch_point(const Geom& g, const DevTables<R>& tb, void* const a[3], int op, double* partial,
                 int npartial, void* stream, LaunchHook hook, void* hctx) {
  Ptr6 pa{};
  for (int i = 0; i < 3; ++i) pa.p[i] = a[i];
  const int threads = 256;
  const int bx = (g.nh + threads - 1) / threads;
  const long long rows = (long long)g.ny * g.nz;
  int by = (int)std::min<long long>(rows, npartial > 0 ? npartial / bx : 65535);
  if (by < 1) by = 1;
  GT_HOOK(kKPoint, true);
  k_point<R><<<dim3(bx, by), threads, 0, (cudaStream_t)stream>>>(pa, tb, g, op, partial);
  GT_HOOK(kKPoint, false);
  int rc = (int)cudaGetLastError();
  if (rc || op != 3) return rc;
  GT_HOOK(kKDiagFinal, true);
  k_final_sum<<<1, kFinalThreads, 0, (cudaStream_t)stream>>>(partial, bx * by, 1, partial + npartial);
  GT_HOOK(kKDiagFinal, false);
  return (int)cudaGetLastError();
}

#ifdef GT_KERNELS_COMMON
int diag_blocks(const Geom& g) {
  const long long rows = (long long)g.ny * g.nz;
  long long b = (rows + 7) / 8;
  return (int)std::min<long long>(b, 152 * 2);
}
#endif

template <typename R>
int launch_diag(const Geom& g, const DevTables<R>& tb, void* const b[3], void* const n1[3],
                double nu, double alpnu, double mu, double alpmu, double* partials, int nblocks,
                double* result, void* stream, LaunchHook hook, void* hctx) {
  int rc0 = set_smem_attrs<R>();
  if (rc0) return rc0;
  Ptr6 pb{}, pn{};
  for (int i = 0; i < 3; ++i) {
    pb.p[i] = b[i];
    pn.p[i] = n1 ? n1[i] : b[i];
  }
  const int nbin = g.nx / 2;
  const int nq = kDiagScalars + 3 * nbin;
  const int smem = 8 * 3 * nbin * (int)sizeof(double);
  GT_HOOK(kKDiag, true);
  k_diag<R><<<nblocks, kDiagThreads, smem, (cudaStream_t)stream>>>(
      pb, pn, tb, g, nu, alpnu, mu, alpmu, n1 != nullptr, partials, nq);
  GT_HOOK(kKDiag, false);
  int rc = (int)cudaGetLastError();
  if (rc) return rc;
  GT_HOOK(kKDiagFinal, true);
  k_final_sum<<<std::max(1, std::min(nq, 1024)), kFinalThreads, 0, (cudaStream_t)stream>>>(partials, nblocks, nq,
                                                                                        result);
  GT_HOOK(kKDiagFinal, false);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_energy(const Geom& g, const DevTables<R>& tb, void* const b[3], int pruned, double* partials,
                  int nblocks, double* result, void* stream, LaunchHook hook, void* hctx) {
  Ptr6 pb{};
  for (int i = 0; i < 3; ++i) pb.p[i] = b[i];
  // one warp per row at a time: one wave of as many blocks as are resident on
  // the device at once (no tail wave), within the partials' capacity
  const long long rows = (long long)g.ny * g.nz;
  const int wave = wave_blocks(k_energy<R>, kDiagThreads, 0);
  nblocks = (int)std::min<long long>({(rows + 7) / 8, wave > 0 ? (long long)wave : 304LL, (long long)nblocks});
  GT_HOOK(kKDiag, true);
  k_energy<R><<<nblocks, kDiagThreads, 0, (cudaStream_t)stream>>>(pb, tb, g, pruned, partials);
  GT_HOOK(kKDiag, false);
  int rc = (int)cudaGetLastError();
  if (rc) return rc;
  GT_HOOK(kKDiagFinal, true);
  k_final_sum<<<3, kFinalThreads, 0, (cudaStream_t)stream>>>(partials, nblocks, 3, result);
  GT_HOOK(kKDiagFinal, false);
  return (int)cudaGetLastError();
}

#ifdef GT_KERNELS_COMMON
void build_ztiles(const Geom& g, const int32_t* xcut, int csize, std::vector<int32_t>& tiles, int tx) {
  const SCfg c = strided_cfg(g.nz, g.nh, 3, csize, csize == 16 ? 512 : 1024);
  const int TX = tx > 0 ? tx : 1 << c.lgTX;
  tiles.clear();
  for (int y = 0; y < g.ny; ++y)
    for (int t = 0; t * TX < xcut[y]; ++t) {
      tiles.push_back(t);
      tiles.push_back(y);
    }
}
#endif

template <typename R>
__global__ void k_count_outside(Ptr6 b, DevTables<R> tb, Geom g, unsigned long long* count) {
  using C = Cplx<R>;
  unsigned long long n = 0;
  const size_t rows = (size_t)g.ny * g.nz;
  for (size_t row = blockIdx.x; row < rows; row += gridDim.x) {
    const int cut = tb.xcut[row];
    for (int X = cut + threadIdx.x; X < g.nh; X += blockDim.x) {
      const size_t o = row * g.nhp + X;
      for (int c = 0; c < 3; ++c) {
        const C v = reinterpret_cast<const C*>(b.at(c))[o];
        if (v.x != (R)0 || v.y != (R)0) ++n;
      }
    }
  }
  if (n) atomicAdd(count, n);
}

template <typename R>
int launch_count_outside(const Geom& g, const DevTables<R>& tb, void* const b[3],
                         unsigned long long* d_count, void* stream) {
  Ptr6 pb{};
  for (int i = 0; i < 3; ++i) pb.p[i] = b[i];
  cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), (cudaStream_t)stream);
  if (e != cudaSuccess) return (int)e;
  const long long rows = (long long)g.ny * g.nz;
  k_count_outside<R><<<(unsigned)std::min<long long>(rows, 152 * 8), 128, 0, (cudaStream_t)stream>>>(
      pb, tb, g, d_count);
  return (int)cudaGetLastError();
}

#ifdef GT_KERNELS_COMMON
const char* kernel_kind_name(int k) {
  static const char* names[kNumKinds] = {"zinv_curl", "yinv", "xcross", "zfwd_epilogue",
                                         "force", "convert", "diag", "diag_final",
                                         "xc2r_xr2c", "pointwise", "yfwd", "zfwd_zinv"};
  return (k >= 0 && k < kNumKinds) ? names[k] : "?";
}
#endif

#define GT_INST(R)                                                                              \
  template int launch_nlt<R>(const Geom&, const DevTables<R>&, void* const*, void* const*,     \
                             void* const*, void* const*, int, int, const PassTuning*, int*,      \
                             void*, LaunchHook, void*);                                         \
  template int launch_rk2_nlts<R>(const Geom&, const DevTables<R>&, void* const*, void* const*, \
                                  void* const*, int, const PassTuning*, int*, void*, LaunchHook,  \
                                  void*, const Batch<R>*);                                     \
  template int launch_count_outside<R>(const Geom&, const DevTables<R>&, void* const*,         \
                                       unsigned long long*, void*);                            \
  template int launch_force<R>(const Geom&, void* const*, const ForceEntry*, int, int, void*,  \
                               LaunchHook, void*);                                              \
  template int launch_force_indexed<R>(const Geom&, void* const*, const ForceEntry*, int,      \
                                       const int*, void*, LaunchHook, void*);                  \
  template int launch_force_batch<R>(const Geom&, void* const*, const Batch<R>&,                \
                                     const ForceEntry*, const int*, int, int, const int*, void*, \
                                     LaunchHook, void*);                                        \
  template int launch_convert<R>(const Geom&, const void*, void*, int, void*, LaunchHook,      \
                                 void*);                                                        \
  template int launch_fft_inv<R>(const Geom&, const DevTables<R>&, void*, void*, void* const*, \
                                 void*, LaunchHook, void*);                                     \
  template int launch_fft_dir<R>(const Geom&, const DevTables<R>&, const void*, void*,         \
                                 void* const*, void*, LaunchHook, void*);                       \
  template int launch_point<R>(const Geom&, const DevTables<R>&, void* const*, int, double*,   \
                               int, void*, LaunchHook, void*);                                  \
  template int launch_energy<R>(const Geom&, const DevTables<R>&, void* const*, int, double*, int, \
                                double*, void*, LaunchHook, void*);                             \
  template int launch_diag<R>(const Geom&, const DevTables<R>&, void* const*, void* const*,    \
                              double, double, double, double, double*, int, double*, void*,    \
                              LaunchHook, void*);

GT_INST(GT_REAL)

}  // namespace gt
