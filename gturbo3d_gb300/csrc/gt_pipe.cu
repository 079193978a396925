// Pipelined y passes: persistent CTAs walk (field, z-plane, x-tile) items;
// thread 0 prefetches the next tiles with TMA tensor loads into a ring of
// shared-memory stages (mbarrier-signalled) while all threads transform the
// current tile, so loads overlap the FFT and its shared-memory exchanges.
//
// Tile = [NY][TX] complex (rows of TX x-columns of one z-plane; TX*element =
// 128 bytes where the shared memory allows).  The TMA box is 16 rows of one
// tile; in the pruned inverse pass only the row ranges holding nonzero data
// (ky with X < xcut0[y] for some column of the tile) are loaded.
#include <algorithm>
#include <cstdio>

#include "gt_fft.cuh"
#include "gt_internal.h"
#include "gt_tma.cuh"

namespace gt {

namespace {

constexpr int kBoxRows = 16;

struct Ptr6p {
  void* p[6];
};

template <typename R> constexpr int pipe_threads() { return sizeof(R) == 8 ? 512 : 1024; }

// Packing of two half spectra into one complex line for the C2R x transform
// (as in k_xcross): entries at kx >= xa are zero.
template <typename R>
__device__ __forceinline__ Cplx<R> pack_c2r_s(const Cplx<R>* X1, const Cplx<R>* X2, int e, int N, int xa) {
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

template <typename R>
__device__ __forceinline__ Cplx<R> xsplit(Cplx<R> a, Cplx<R> b, bool first, R s) {
  using C = Cplx<R>;
  return first ? C{(a.x + b.x) * s, (a.y - b.y) * s} : C{(a.y + b.y) * s, (b.x - a.x) * s};
}

// Rows of the tile starting at column x0 that hold data in the pruned inverse
// pass: y in [0, c) and [ny - c + 1, ny), with c = #{y <= ny/2 : xcut0[y] > x0}.
__device__ __forceinline__ int active_rows(const int32_t* __restrict__ xcut0, int ny, int x0) {
  int lo = 0, hi = ny / 2 + 1;   // xcut0 is non-increasing on [0, ny/2]
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (xcut0[mid] > x0) lo = mid + 1; else hi = mid;
  }
  return lo;
}

template <typename R, int SIGN>
__global__ void __launch_bounds__(pipe_threads<R>())
k_ypipe(const __grid_constant__ PipeMaps maps, Ptr6p f, Geom g, const void* twv, int nf, int ntx,
        int lgTX, int nstage, int xlim, int ymask, const int32_t* __restrict__ xcut0, int* err) {
  using C = Cplx<R>;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int TX = 1 << lgTX;
  const int L = g.ny, lgL = g.lny, T = L >> 3;
  const int tileElems = L * TX;
  C* stages = reinterpret_cast<C*>(smraw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smraw + (size_t)nstage * tileElems * sizeof(C));
  const int x = threadIdx.x & (TX - 1), t = threadIdx.x >> lgTX;
  const long long nitems = (long long)nf * g.nz * ntx;
  const long long G = gridDim.x;
  const uint32_t boxBytes = (uint32_t)(kBoxRows * TX * sizeof(C));
  const size_t plane = (size_t)g.ny * g.nhp;

  if (threadIdx.x == 0) {
    for (int s = 0; s < nstage; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // thread 0: load item w into stage s
  auto issue = [&](long long w, int s) {
    const int tx = (int)(w % ntx);
    const long long r = w / ntx;
    const int z = (int)(r % g.nz), fi = (int)(r / g.nz);
    const int x0 = tx * TX;
    C* tile = stages + (size_t)s * tileElems;
    const CUtensorMap* map = &maps.y[fi];
    int nb1, b2lo;   // boxes [0, nb1) and [b2lo, L/16)
    if (ymask == 1) {
      const int c = active_rows(xcut0, g.ny, x0);
      nb1 = (c + kBoxRows - 1) / kBoxRows;
      const int y2 = L - c + 1;                   // first active row of the negative half
      b2lo = c > 1 ? y2 / kBoxRows : L / kBoxRows;
      if (b2lo < nb1) b2lo = nb1;
    } else {
      nb1 = L / kBoxRows;
      b2lo = nb1;
    }
    const int nboxes = nb1 + (L / kBoxRows - b2lo);
    mbar_arrive_expect_tx(&bars[s], (uint32_t)nboxes * boxBytes);
    for (int b = 0; b < nb1; ++b)
      tma_load_3d(tile + b * kBoxRows * TX, map, 2 * x0, b * kBoxRows, z, &bars[s]);
    for (int b = b2lo; b < L / kBoxRows; ++b)
      tma_load_3d(tile + b * kBoxRows * TX, map, 2 * x0, b * kBoxRows, z, &bars[s]);
  };

  long long w = blockIdx.x;
  if (threadIdx.x == 0)
    for (int s = 0; s < nstage - 1; ++s)
      if (w + s * G < nitems) issue(w + s * G, s);
  int it = 0;
  long long consumed_upto = -1;   // iterations whose stage has been waited on
  bool failed = false;
  for (; w < nitems; w += G, ++it) {
    const int s = it % nstage;
    if (threadIdx.x == 0) {
      const long long wn = w + (long long)(nstage - 1) * G;
      if (wn < nitems) {
        fence_proxy_async_smem();
        issue(wn, (it + nstage - 1) % nstage);
      }
    }
    const bool ok = mbar_wait(&bars[s], (uint32_t)((it / nstage) & 1));
    if (!__syncthreads_and(ok)) {
      failed = true;
      break;
    }
    consumed_upto = it;
    const int tx = (int)(w % ntx);
    const long long r = w / ntx;
    const int z = (int)(r % g.nz), fi = (int)(r / g.nz);
    const int X = tx * TX + x;
    const bool valid = X < xlim;
    C* tile = stages + (size_t)s * tileElems;
    C v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = t + i * T;
      const bool ld = valid && (ymask != 1 || X < xcut0[e]);
      v[i] = ld ? tile[e * TX + x] : C{0, 0};
    }
    __syncthreads();
    fft_line<SIGN, R>(v, t, lgL, reinterpret_cast<const C*>(twv), tile, StridedIdx{TX, x});
    if (valid) {
      C* p = reinterpret_cast<C*>(f.p[fi]) + (size_t)z * plane + X;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = t + i * T;
        if (ymask != 2 || X < xcut0[e]) p[(size_t)e * g.nhp] = v[i];
      }
    }
    if (lgL == 3) __syncthreads();   // fft_line had no barrier: free the stage before reuse
  }
  if (failed && threadIdx.x == 0) {
    raise_error(err, GT_ETIMEOUT);
    // wait (bounded) for the loads this CTA issued and did not consume
    for (int k = 1; k <= nstage; ++k) {
      const long long itk = consumed_upto + k;
      const long long wk = blockIdx.x + itk * G;
      if (wk < nitems) mbar_wait(&bars[itk % nstage], (uint32_t)((itk / nstage) & 1));
    }
  }
}

// Pipelined pass 5: forward z transform of w[0..2] and the spectral epilogue
// (Coriolis, invcurl, trunc, step1/step2).  Items are (x-tile, y) column
// blocks (the pruned tile list, or the full grid); a stage holds the three
// fields' [NZ][TX] tiles, loaded with TMA boxes of up to 256 z-planes.
template <typename R>
__global__ void __launch_bounds__(pipe_threads<R>() / 2)
k_zpipe_epi(const __grid_constant__ PipeMaps maps, Ptr6p bc, Ptr6p out, DevTables<R> tb, Geom g,
            int lgTX, int nstage, int mode, int pruned, int ntx, int* err) {
  using C = Cplx<R>;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int TX = 1 << lgTX;
  const int L = g.nz, lgL = g.lnz, T = L >> 3;
  const int fieldElems = L * TX, stageElems = 3 * fieldElems;
  C* stages = reinterpret_cast<C*>(smraw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smraw + (size_t)nstage * stageElems * sizeof(C));
  const int x = threadIdx.x & (TX - 1), t = threadIdx.x >> lgTX;
  const long long nitems = pruned ? (long long)tb.nztiles_p : (long long)ntx * g.ny;
  const long long G = gridDim.x;
  const int bz = L < 256 ? L : 256;
  const uint32_t boxBytes = (uint32_t)(bz * TX * sizeof(C));
  const size_t plane = (size_t)g.ny * g.nhp;
  const StridedIdx idx{TX, x};
  const C* tw = reinterpret_cast<const C*>(tb.twz);

  if (threadIdx.x == 0) {
    for (int s = 0; s < nstage; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto item = [&](long long w, int& tile, int& y) {
    if (pruned) {
      tile = tb.ztiles_p[2 * w];
      y = tb.ztiles_p[2 * w + 1];
    } else {
      tile = (int)(w % ntx);
      y = (int)(w / ntx);
    }
  };
  auto issue = [&](long long w, int s) {
    int tile, y;
    item(w, tile, y);
    C* st = stages + (size_t)s * stageElems;
    const int nb = L / bz;
    mbar_arrive_expect_tx(&bars[s], 3u * nb * boxBytes);
    for (int f = 0; f < 3; ++f)
      for (int b = 0; b < nb; ++b)
        tma_load_3d(st + f * fieldElems + b * bz * TX, &maps.z[f], 2 * tile * TX, y, b * bz, &bars[s]);
  };

  long long w = blockIdx.x;
  if (threadIdx.x == 0)
    for (int s = 0; s < nstage - 1; ++s)
      if (w + s * G < nitems) issue(w + s * G, s);
  int it = 0;
  long long consumed_upto = -1;
  bool failed = false;
  for (; w < nitems; w += G, ++it) {
    const int s = it % nstage;
    if (threadIdx.x == 0) {
      const long long wn = w + (long long)(nstage - 1) * G;
      if (wn < nitems) {
        fence_proxy_async_smem();
        issue(wn, (it + nstage - 1) % nstage);
      }
    }
    const bool ok = mbar_wait(&bars[s], (uint32_t)((it / nstage) & 1));
    if (!__syncthreads_and(ok)) {
      failed = true;
      break;
    }
    consumed_upto = it;
    int tile, y;
    item(w, tile, y);
    const int X = tile * TX + x;
    const bool valid = X < (pruned ? tb.xcut[y] : g.nh);
    C* st = stages + (size_t)s * stageElems;
    C v[8];
    for (int f = 0; f < 3; ++f) {
      C* S = st + f * fieldElems;
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = S[idx(t + i * T)];
      __syncthreads();
      fft_line<-1, R>(v, t, lgL, tw, S, idx);
#pragma unroll
      for (int i = 0; i < 8; ++i) S[idx(t + i * T)] = v[i];
    }
    if (valid) {
      const size_t base = (size_t)y * g.nhp + X;
      const R kx = tb.fkx[X], ky = tb.fky[y], kxs = tb.fkxs[X], kys = tb.fkys[y];
      const C* b0p = reinterpret_cast<const C*>(bc.p[0]);
      const C* b1p = reinterpret_cast<const C*>(bc.p[1]);
      const C* b2p = reinterpret_cast<const C*>(bc.p[2]);
      C* o0 = reinterpret_cast<C*>(out.p[0]);
      C* o1 = reinterpret_cast<C*>(out.p[1]);
      C* o2 = reinterpret_cast<C*>(out.p[2]);
      for (int i = 0; i < 8; ++i) {
        const int z = t + i * T;
        const bool kept = X < tb.xcut[(size_t)z * g.ny + y];
        if (pruned && !kept) continue;
        const size_t o = (size_t)z * plane + base;
        const C n0 = st[idx(z)], n1 = st[fieldElems + idx(z)], n2 = st[2 * fieldElems + idx(z)];
        const C b0 = b0p[o], b1 = b1p[o], b2 = b2p[o];
        const R okz = tb.omega * tb.fkz[z];
        const C a0{n0.x - okz * b0.y, n0.y + okz * b0.x};
        const C a1{n1.x - okz * b1.y, n1.y + okz * b1.x};
        const C a2{n2.x - okz * b2.y, n2.y + okz * b2.x};
        const bool zero_mode = (X == 0) && (y == 0) && (z == 0);
        const R k2 = (kxs + kys) + tb.fkzs[z];
        C r0 = a0, r1 = a1, r2 = a2;
        if (!zero_mode) {
          const R ik2 = (R)1 / k2;
          const R qx = kx * ik2, qy = ky * ik2, qz = tb.fkz[z] * ik2;
          r0 = C{-qy * a2.y + qz * a1.y, qy * a2.x - qz * a1.x};
          r1 = C{-qz * a0.y + qx * a2.y, qz * a0.x - qx * a2.x};
          r2 = C{-qx * a1.y + qy * a0.y, qx * a1.x - qy * a0.x};
        }
        if (tb.truncate && (zero_mode || !kept)) {
          r0 = C{0, 0}; r1 = C{0, 0}; r2 = C{0, 0};
        }
        if (mode == kNltOnly) {
          o0[o] = r0; o1[o] = r1; o2[o] = r2;
        } else {
          const R e = tb.emk_by_k2 ? tb.emk[(int)k2] : tb.emk[((size_t)z * g.ny + y) * g.nh + X];
          C s0, s1, s2;
          if (mode == kStage1) {
            const R d = tb.dt2;
            s0 = C{e * (b0.x + d * r0.x), e * (b0.y + d * r0.y)};
            s1 = C{e * (b1.x + d * r1.x), e * (b1.y + d * r1.y)};
            s2 = C{e * (b2.x + d * r2.x), e * (b2.y + d * r2.y)};
          } else {
            const R d = tb.dt;
            s0 = C{e * (e * b0.x + d * r0.x), e * (e * b0.y + d * r0.y)};
            s1 = C{e * (e * b1.x + d * r1.x), e * (e * b1.y + d * r1.y)};
            s2 = C{e * (e * b2.x + d * r2.x), e * (e * b2.y + d * r2.y)};
          }
          if (zero_mode) {
            s0 = C{0, 0}; s1 = C{0, 0}; s2 = C{0, 0};
          }
          o0[o] = s0; o1[o] = s1; o2[o] = s2;
        }
      }
    }
    __syncthreads();   // the stage is free for the next load
  }
  if (failed && threadIdx.x == 0) {
    raise_error(err, GT_ETIMEOUT);
    for (int k = 1; k <= nstage; ++k) {
      const long long itk = consumed_upto + k;
      const long long wk = blockIdx.x + itk * G;
      if (wk < nitems) mbar_wait(&bars[itk % nstage], (uint32_t)((itk / nstage) & 1));
    }
  }
}

// Pipelined pass 3 (x transforms with u x w): persistent CTAs walk groups of
// P row pairs; thread 0 prefetches the next group's 12*P half-spectrum row
// segments (6 fields x 2 rows x the first `seg` columns, seg*element a
// multiple of 16 bytes) with 1D bulk copies into a staging ring, so the C2R
// packing reads shared memory.  The transforms and the u x w product are
// those of k_xcross.
template <typename R>
__global__ void __launch_bounds__(pipe_threads<R>() / 2)
k_xpipe(Ptr6p w, Geom g, const void* twv, int P, int sh, R shalf, int xa, int seg, int nstage, int* err) {
  using C = Cplx<R>;
  extern __shared__ __align__(128) unsigned char smraw[];
  const int N = g.nx, lgN = g.lnx, lgT = lgN - 3, T = 1 << lgT;
  const int LP = N + (N >> sh);
  const int stageElems = 12 * P * seg;
  C* stages = reinterpret_cast<C*>(smraw);
  C* sm = stages + (size_t)nstage * stageElems;              // 6P FFT lines
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + (size_t)6 * P * LP);
  const int gid = threadIdx.x >> lgT, t = threadIdx.x & (T - 1);
  const int p = gid / 3, q = gid - 3 * p;
  const C* tw = reinterpret_cast<const C*>(twv);
  const size_t nhp = g.nhp;
  const long long nitems = (long long)g.ny * g.nz / 2 / P;
  const long long G = gridDim.x;
  const uint32_t segBytes = (uint32_t)(seg * sizeof(C));

  if (threadIdx.x == 0) {
    for (int s = 0; s < nstage; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto issue = [&](long long item, int s) {
    C* st = stages + (size_t)s * stageElems;
    mbar_arrive_expect_tx(&bars[s], 12u * P * segBytes);
    for (int pp = 0; pp < P; ++pp)
      for (int f = 0; f < 6; ++f)
        for (int r = 0; r < 2; ++r) {
          const size_t row = 2 * ((size_t)item * P + pp) + r;
          bulk_load_1d(st + ((pp * 6 + f) * 2 + r) * seg, reinterpret_cast<const C*>(w.p[f]) + row * nhp,
                       segBytes, &bars[s]);
        }
  };

  long long item = blockIdx.x;
  if (threadIdx.x == 0)
    for (int s = 0; s < nstage - 1; ++s)
      if (item + s * G < nitems) issue(item + s * G, s);
  int it = 0;
  long long consumed_upto = -1;
  bool failed = false;
  for (; item < nitems; item += G, ++it) {
    const int s = it % nstage;
    if (threadIdx.x == 0) {
      const long long wn = item + (long long)(nstage - 1) * G;
      if (wn < nitems) {
        fence_proxy_async_smem();
        issue(wn, (it + nstage - 1) % nstage);
      }
    }
    const bool ok = mbar_wait(&bars[s], (uint32_t)((it / nstage) & 1));
    if (!__syncthreads_and(ok)) {
      failed = true;
      break;
    }
    consumed_upto = it;
    const C* st = stages + (size_t)s * stageElems;
    const size_t pair = (size_t)item * P + p;
    C v[8];
    for (int r = 0; r < 2; ++r) {
      const C* X1 = st + ((p * 6 + 2 * q) * 2 + r) * seg;
      const C* X2 = st + ((p * 6 + 2 * q + 1) * 2 + r) * seg;
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = pack_c2r_s<R>(X1, X2, t + i * T, N, xa);
      const PaddedIdx idx{(p * 6 + r * 3 + q) * LP, sh};
      fft_line<+1, R>(v, t, lgN, tw, sm, idx);
#pragma unroll
      for (int i = 0; i < 8; ++i) sm[idx(t + i * T)] = v[i];
    }
    __syncthreads();
    for (int n = threadIdx.x; n < P * N; n += blockDim.x) {
      const int pp = n >> lgN, e = n & (N - 1);
      const int o = pp * 6 * LP + e + (e >> sh);
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
      const PaddedIdx idx{line * LP, sh};
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = sm[idx(t + i * T)];
      __syncthreads();
      fft_line<-1, R>(v, t, lgN, tw, sm, idx);
#pragma unroll
      for (int i = 0; i < 8; ++i) sm[idx(t + i * T)] = v[i];
    }
    __syncthreads();
    {
      const int lineA = p * 6 + (q == 2 ? 1 : 0), lineB = p * 6 + (q == 2 ? 1 : 3);
      C* out = reinterpret_cast<C*>(w.p[q]);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int o = (r == 0 ? lineA : lineB) * LP;
        const bool first = (q == 0) || (q == 2 && r == 0);
        C* orow = out + (2 * pair + r) * nhp;
        for (int k = t; k < xa; k += T) {
          const int kb = (N - k) & (N - 1);
          const C a = sm[o + k + (k >> sh)], b = sm[o + kb + (kb >> sh)];
          orow[k] = xsplit<R>(a, b, first, shalf);
        }
      }
    }
    __syncthreads();   // the FFT lines are reused by the next item
  }
  if (failed && threadIdx.x == 0) {
    raise_error(err, GT_ETIMEOUT);
    for (int k = 1; k <= nstage; ++k) {
      const long long itk = consumed_upto + k;
      const long long wk = blockIdx.x + itk * G;
      if (wk < nitems) mbar_wait(&bars[itk % nstage], (uint32_t)((itk / nstage) & 1));
    }
  }
}

}  // namespace

PFN_encodeTiled get_encode_tiled() {
  static PFN_encodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_encodeTiled>(p);
  }
  return fn;
}

int ypipe_tx(const Geom& g, int csize) {
  int TX = 128 / csize;
  const int maxt = csize == 16 ? 512 : 1024;
  while (TX > 2 && (g.ny / 8) * TX > maxt) TX >>= 1;
  return TX;
}

int make_ypipe_maps(const Geom& g, int csize, void* const w[6], PipeMaps& pm) {
  PFN_encodeTiled enc = get_encode_tiled();
  if (!enc) return (int)cudaErrorNotSupported;
  const int TX = ypipe_tx(g, csize);
  const size_t esz = csize / 2;
  for (int f = 0; f < 6; ++f) {
    cuuint64_t dims[3] = {(cuuint64_t)2 * g.nhp, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    cuuint64_t strides[2] = {(cuuint64_t)2 * g.nhp * esz, (cuuint64_t)2 * g.nhp * esz * g.ny};
    cuuint32_t box[3] = {(cuuint32_t)(2 * TX), (cuuint32_t)kBoxRows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(&pm.y[f], esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                     3, w[f], dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return (int)cudaErrorInvalidValue;
  }
  pm.ytx = TX;
  const int ZTX = zpipe_tx(g, csize);
  const cuuint32_t bz = g.nz < 256 ? (cuuint32_t)g.nz : 256u;
  for (int f = 0; f < 3 && ZTX > 0; ++f) {
    cuuint64_t dims[3] = {(cuuint64_t)2 * g.nhp, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
    cuuint64_t strides[2] = {(cuuint64_t)2 * g.nhp * esz, (cuuint64_t)2 * g.nhp * esz * g.ny};
    cuuint32_t box[3] = {(cuuint32_t)(2 * ZTX), 1u, bz};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(&pm.z[f], esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                     3, w[f], dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return (int)cudaErrorInvalidValue;
  }
  pm.ztx = ZTX;
  pm.valid = 1;
  return 0;
}

int zpipe_tx(const Geom& g, int csize) {
  // three fields per stage, two stages, within the per-block shared memory;
  // 0 (use the one-tile-per-CTA pass) when that leaves fewer than 4 columns
  int TX = 128 / csize;
  while (TX > 2 && ((size_t)6 * g.nz * TX * csize > 200 * 1024 || (g.nz / 8) * TX > (csize == 16 ? 256 : 512)))
    TX >>= 1;
  return TX >= 4 ? TX : 0;
}

template <typename R>
int launch_zpipe_epi(const Geom& g, const DevTables<R>& tb, const PipeMaps& pm, void* const bcor[3],
                     void* const out[3], int mode, int pruned, int* err, void* stream, LaunchHook hook,
                     void* hctx) {
  using C = Cplx<R>;
  const int TX = pm.ztx;
  const int lgTX = [&] { int l = 0; while ((1 << l) < TX) ++l; return l; }();
  const int threads = (g.nz / 8) * TX;
  const size_t stageBytes = (size_t)3 * g.nz * TX * sizeof(C);
  int dev = 0, optin = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nstage = (int)std::min<size_t>(3, (optin - 64) / stageBytes);
  if (nstage < 2) return (int)cudaErrorInvalidConfiguration;
  const size_t smem = nstage * stageBytes + 64;
  const int ntx = (g.nh + TX - 1) / TX;
  Ptr6p pb{}, po{};
  for (int i = 0; i < 3; ++i) {
    pb.p[i] = bcor[i];
    po.p[i] = out[i];
  }
  cudaError_t e = cudaFuncSetAttribute(k_zpipe_epi<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_zpipe_epi<R>, threads, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) per_sm = 1;
  const long long nitems = pruned ? (long long)tb.nztiles_p : (long long)ntx * g.ny;
  const int grid = (int)std::min<long long>(nitems, (long long)nsm * per_sm);
  if (hook) hook(hctx, kKZFwdEpi, true);
  k_zpipe_epi<R><<<grid, threads, smem, (cudaStream_t)stream>>>(pm, pb, po, tb, g, lgTX, nstage, mode, pruned,
                                                               ntx, err);
  if (hook) hook(hctx, kKZFwdEpi, false);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_xpipe(const Geom& g, void* const w[6], const void* twx, int xa, int pairs, int nstage,
                 int* err, void* stream, LaunchHook hook, void* hctx) {
  using C = Cplx<R>;
  const int sh = sizeof(R) == 8 ? 3 : 4;
  const int LP = g.nx + (g.nx >> sh);
  const int per16 = 16 / (int)sizeof(C) > 0 ? 16 / (int)sizeof(C) : 1;
  int seg = (xa + per16 - 1) / per16 * per16;
  if (seg > g.nhp) seg = g.nhp;
  const long long npairs = (long long)g.ny * g.nz / 2;
  int P = pairs > 0 ? pairs : 1;
  while (P > 1 && npairs % P) P >>= 1;
  const int threads = 3 * P * (g.nx / 8);
  if (threads > pipe_threads<R>() / 2) return (int)cudaErrorInvalidConfiguration;
  const size_t smem = (size_t)nstage * 12 * P * seg * sizeof(C) + (size_t)6 * P * LP * sizeof(C) + 64;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaFuncSetAttribute(k_xpipe<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_xpipe<R>, threads, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) return (int)cudaErrorInvalidConfiguration;
  const long long nitems = npairs / P;
  const int grid = (int)std::min<long long>(nitems, (long long)nsm * per_sm);
  Ptr6p pw{};
  for (int i = 0; i < 6; ++i) pw.p[i] = w[i];
  const R shalf = (R)(0.5 / ((double)g.nx * g.ny * g.nz));
  if (hook) hook(hctx, kKXCross, true);
  k_xpipe<R><<<grid, threads, smem, (cudaStream_t)stream>>>(pw, g, twx, P, sh, shalf, xa, seg, nstage, err);
  if (hook) hook(hctx, kKXCross, false);
  return (int)cudaGetLastError();
}

template int launch_xpipe<float>(const Geom&, void* const*, const void*, int, int, int, int*, void*,
                                 LaunchHook, void*);
template int launch_xpipe<double>(const Geom&, void* const*, const void*, int, int, int, int*, void*,
                                  LaunchHook, void*);

template int launch_zpipe_epi<float>(const Geom&, const DevTables<float>&, const PipeMaps&, void* const*,
                                     void* const*, int, int, int*, void*, LaunchHook, void*);
template int launch_zpipe_epi<double>(const Geom&, const DevTables<double>&, const PipeMaps&, void* const*,
                                      void* const*, int, int, int*, void*, LaunchHook, void*);

template <typename R>
int launch_ypipe(const Geom& g, const PipeMaps& pm, void* const* fields, int nf, const void* tw,
                 int sign, int xlim, int ymask, const int32_t* xcut0, int* err, void* stream,
                 LaunchHook hook, void* hctx) {
  using C = Cplx<R>;
  const int TX = pm.ytx;
  const int lgTX = [&] { int l = 0; while ((1 << l) < TX) ++l; return l; }();
  const int threads = (g.ny / 8) * TX;
  const size_t tileBytes = (size_t)g.ny * TX * sizeof(C);
  int dev = 0, optin = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int nstage = (int)std::min<size_t>(3, (optin - 64) / tileBytes);
  if (nstage < 2) return (int)cudaErrorInvalidConfiguration;
  const size_t smem = nstage * tileBytes + 64;
  const int ntx = (xlim + TX - 1) / TX;
  Ptr6p pf{};
  for (int i = 0; i < nf; ++i) pf.p[i] = fields[i];
  auto kern = sign > 0 ? k_ypipe<R, 1> : k_ypipe<R, -1>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
  if (e != cudaSuccess) return (int)e;
  if (per_sm < 1) per_sm = 1;
  const long long nitems = (long long)nf * g.nz * ntx;
  const int grid = (int)std::min<long long>(nitems, (long long)nsm * per_sm);
  const int kind = sign > 0 ? kKYPass : kKYFwd;
  if (hook) hook(hctx, kind, true);
  kern<<<grid, threads, smem, (cudaStream_t)stream>>>(pm, pf, g, tw, nf, ntx, lgTX, nstage, xlim, ymask,
                                                     xcut0, err);
  if (hook) hook(hctx, kind, false);
  return (int)cudaGetLastError();
}

// Self-test of the bounded-wait path: one thread waits on an mbarrier that
// nothing arrives at (no copy is issued), gives up after `limit` polls and
// records GT_ETIMEOUT in the error flag, exactly as a pipelined pass does when
// its copies never land.  Nothing is in flight when it returns.
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

template int launch_ypipe<float>(const Geom&, const PipeMaps&, void* const*, int, const void*, int, int,
                                 int, const int32_t*, int*, void*, LaunchHook, void*);
template int launch_ypipe<double>(const Geom&, const PipeMaps&, void* const*, int, const void*, int, int,
                                  int, const int32_t*, int*, void*, LaunchHook, void*);

}  // namespace gt
