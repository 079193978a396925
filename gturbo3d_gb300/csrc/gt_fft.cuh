// Device FFT building blocks: complex arithmetic, radix-2/4/8 butterflies and
// a Stockham line transform in which each thread holds 8 elements.
//
// Line transform convention.  A line of length L = 2^lgL (8 <= L <= 1024) is
// transformed by L/8 threads t = 0..L/8-1.  On entry thread t holds
// v[i] = x[t + i L/8] (i = 0..7); on exit it holds X[t + i L/8] in natural
// order, so the first stage can be fed from global memory and the last stage
// can store to global memory without a shared-memory round trip.  Stages use
// radix 8 while at least three factors of two remain, then one radix-4 or
// radix-2 stage.  A stage with radix r and Ns = product of earlier radices does
// 8/r butterflies b = t + m L/8 per thread; butterfly b reads registers
// m + j (8/r), multiplies input j by W_{Ns r}^{j (b mod Ns)} and writes output
// j to position (b div Ns) Ns r + (b mod Ns) + j Ns.
//
// SIGN = -1 is the forward transform X_k = sum x_n e^{-2 pi i k n / L}
// (numpy and cuFFT convention); SIGN = +1 the unnormalised inverse.
#pragma once

#include <cuda_runtime.h>

namespace gt {

template <typename R> struct CplxOf;
template <> struct CplxOf<float> { using type = float2; };
template <> struct CplxOf<double> { using type = double2; };
template <typename R> using Cplx = typename CplxOf<R>::type;

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return C{a.x + b.x, a.y + b.y}; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return C{a.x - b.x, a.y - b.y}; }

// FP32 complex add/sub as one paired instruction (add.rn.f32x2 / sub.rn.f32x2,
// sm_100 and later): each lane is rounded to nearest as two add.rn.f32 would
// be, so results are bit-identical and the butterflies issue half the adds.
#ifndef GT_NO_F32X2
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "add.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
#endif

// Two complex values of adjacent x columns, transformed together by one
// thread of a strided pass (a 16-byte load or store for FP32): the twiddle
// and the index arithmetic of a stage serve both.
template <typename R> struct __align__(2 * sizeof(Cplx<R>)) CPair {
  Cplx<R> a, b;
};
template <typename R> __device__ __forceinline__ CPair<R> cadd(CPair<R> p, CPair<R> q) {
  return CPair<R>{cadd(p.a, q.a), cadd(p.b, q.b)};
}
template <typename R> __device__ __forceinline__ CPair<R> csub(CPair<R> p, CPair<R> q) {
  return CPair<R>{csub(p.a, q.a), csub(p.b, q.b)};
}

// Three complex values at the same position of three lines transformed
// together by one thread (the x pass's three packed lines of a row): the
// stage's twiddles, index arithmetic and barriers serve all three, and the
// three dependency chains interleave.
template <typename R> struct CTrip {
  Cplx<R> a, b, c;
};
template <typename R> __device__ __forceinline__ CTrip<R> cadd(CTrip<R> p, CTrip<R> q) {
  return CTrip<R>{cadd(p.a, q.a), cadd(p.b, q.b), cadd(p.c, q.c)};
}
template <typename R> __device__ __forceinline__ CTrip<R> csub(CTrip<R> p, CTrip<R> q) {
  return CTrip<R>{csub(p.a, q.a), csub(p.b, q.b), csub(p.c, q.c)};
}

// a * W4^{SIGN}: the forward transform multiplies by -i, the inverse by +i.
template <int SIGN, typename C> __device__ __forceinline__ C rot90(C a) {
  return SIGN < 0 ? C{a.y, -a.x} : C{-a.y, a.x};
}

// a * w (forward) or a * conj(w) (inverse) for a table entry w = e^{-2 pi i m/L}.
template <int SIGN, typename C> __device__ __forceinline__ C twmul(C a, C w) {
  if (SIGN < 0) return C{a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x};
  return C{a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y};
}

template <int SIGN, typename R> __device__ __forceinline__ CPair<R> rot90(CPair<R> p) {
  return CPair<R>{rot90<SIGN>(p.a), rot90<SIGN>(p.b)};
}
template <int SIGN, typename R> __device__ __forceinline__ CPair<R> twmul(CPair<R> p, Cplx<R> w) {
  return CPair<R>{twmul<SIGN>(p.a, w), twmul<SIGN>(p.b, w)};
}
template <int SIGN, typename R> __device__ __forceinline__ CTrip<R> rot90(CTrip<R> p) {
  return CTrip<R>{rot90<SIGN>(p.a), rot90<SIGN>(p.b), rot90<SIGN>(p.c)};
}
template <int SIGN, typename R> __device__ __forceinline__ CTrip<R> twmul(CTrip<R> p, Cplx<R> w) {
  return CTrip<R>{twmul<SIGN>(p.a, w), twmul<SIGN>(p.b, w), twmul<SIGN>(p.c, w)};
}

template <typename C> __device__ __forceinline__ void dft2(C& a, C& b) {
  const C t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <int SIGN, typename C> __device__ __forceinline__ void dft4(C& x0, C& x1, C& x2, C& x3) {
  const C s0 = cadd(x0, x2), d0 = csub(x0, x2);
  const C s1 = cadd(x1, x3), d1 = rot90<SIGN>(csub(x1, x3));
  x0 = cadd(s0, s1);
  x2 = csub(s0, s1);
  x1 = cadd(d0, d1);
  x3 = csub(d0, d1);
}

// Multiplication by W8 = (1 -+ i)/sqrt2 and W8^3 = (-1 -+ i)/sqrt2 (upper sign
// forward), and the radix-2 combination e +- o of such a product written
// component-wise so that the products fuse into FMAs.
template <int SIGN, typename R> __device__ __forceinline__ Cplx<R> w8_1(Cplx<R> o) {
  const R c = (R)0.70710678118654752440;
  return SIGN < 0 ? Cplx<R>{c * (o.x + o.y), c * (o.y - o.x)} : Cplx<R>{c * (o.x - o.y), c * (o.x + o.y)};
}
template <int SIGN, typename R> __device__ __forceinline__ Cplx<R> w8_3(Cplx<R> o) {
  const R c = (R)0.70710678118654752440;
  return SIGN < 0 ? Cplx<R>{c * (o.y - o.x), -c * (o.x + o.y)} : Cplx<R>{-c * (o.x + o.y), c * (o.x - o.y)};
}
template <typename C> __device__ __forceinline__ C fadd(C e, C o) { return C{e.x + o.x, e.y + o.y}; }
template <typename C> __device__ __forceinline__ C fsub(C e, C o) { return C{e.x - o.x, e.y - o.y}; }
template <int SIGN, typename R> __device__ __forceinline__ CPair<R> w8_1(CPair<R> p) {
  return CPair<R>{w8_1<SIGN, R>(p.a), w8_1<SIGN, R>(p.b)};
}
template <int SIGN, typename R> __device__ __forceinline__ CPair<R> w8_3(CPair<R> p) {
  return CPair<R>{w8_3<SIGN, R>(p.a), w8_3<SIGN, R>(p.b)};
}
template <typename R> __device__ __forceinline__ CPair<R> fadd(CPair<R> e, CPair<R> o) {
  return CPair<R>{fadd(e.a, o.a), fadd(e.b, o.b)};
}
template <typename R> __device__ __forceinline__ CPair<R> fsub(CPair<R> e, CPair<R> o) {
  return CPair<R>{fsub(e.a, o.a), fsub(e.b, o.b)};
}
template <int SIGN, typename R> __device__ __forceinline__ CTrip<R> w8_1(CTrip<R> p) {
  return CTrip<R>{w8_1<SIGN, R>(p.a), w8_1<SIGN, R>(p.b), w8_1<SIGN, R>(p.c)};
}
template <int SIGN, typename R> __device__ __forceinline__ CTrip<R> w8_3(CTrip<R> p) {
  return CTrip<R>{w8_3<SIGN, R>(p.a), w8_3<SIGN, R>(p.b), w8_3<SIGN, R>(p.c)};
}
template <typename R> __device__ __forceinline__ CTrip<R> fadd(CTrip<R> e, CTrip<R> o) {
  return CTrip<R>{fadd(e.a, o.a), fadd(e.b, o.b), fadd(e.c, o.c)};
}
template <typename R> __device__ __forceinline__ CTrip<R> fsub(CTrip<R> e, CTrip<R> o) {
  return CTrip<R>{fsub(e.a, o.a), fsub(e.b, o.b), fsub(e.c, o.c)};
}

// 8-point DFT in natural order: two 4-point DFTs of the even and odd inputs,
// the odd outputs rotated by W8^q, then one radix-2 layer.  C is a complex
// value or a CPair of two.
template <int SIGN, typename R, typename C> __device__ __forceinline__ void dft8(C v[8]) {
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<SIGN>(e0, e1, e2, e3);
  dft4<SIGN>(o0, o1, o2, o3);
  o1 = w8_1<SIGN, R>(o1);
  o2 = rot90<SIGN>(o2);
  o3 = w8_3<SIGN, R>(o3);
  v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
  v[1] = fadd(e1, o1); v[5] = fsub(e1, o1);
  v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
  v[3] = fadd(e3, o3); v[7] = fsub(e3, o3);
}

// Offset, within the per-stage twiddle table, of the stage that starts after
// 2^lgns points: every earlier stage but the first (radix r, Ns points
// before it) holds (r - 1) Ns entries tw[j k L / (Ns r)] in [j - 1][k] order.
constexpr int tw_stage_offset(int lgl, int lgns) {
  int off = 0;
  for (int s = 0; s < lgns;) {
    const int lr = lgl - s >= 3 ? 3 : lgl - s;
    if (s > 0) off += ((1 << lr) - 1) << s;
    s += lr;
  }
  return off;
}

// The same transform with the line length fixed at compile time: the stage
// sequence unrolls (template recursion), so radices, strides, masks and
// shifts are constants and no per-stage control flow or index arithmetic is
// left at run time.  Twiddles come from the per-stage table stored after the
// L entries of the full table (`tw + L`), where the lanes of a warp read
// consecutive entries.
// The twiddles one thread applies in the stage that starts after 2^LGNS
// points: radix 8: 7 for its butterfly; radix 4: 3 for each of its 2
// butterflies; radix 2: 1 for each of its 4.  Loaded a stage ahead, so that
// their latency overlaps the previous stage's butterflies and exchange.
template <typename R, int LGL, int LGNS> struct StageTw {
  static constexpr int REM = LGL - LGNS;
  static constexpr int LR = REM >= 3 ? 3 : REM;
  static constexpr int NS = 1 << LGNS;
  static constexpr int T = 1 << (LGL - 3);
  static constexpr int N = LGNS == 0 ? 1 : (LR == 3 ? 7 : (LR == 2 ? 6 : 4));
  Cplx<R> w[N];
  __device__ __forceinline__ void load(int t, const Cplx<R>* __restrict__ tw) {
    if constexpr (LGNS > 0) {
      const Cplx<R>* tws = tw + (1 << LGL) + tw_stage_offset(LGL, LGNS);
      if constexpr (LR == 3) {
        const int k = t & (NS - 1);
#pragma unroll
        for (int j = 1; j < 8; ++j) w[j - 1] = __ldg(&tws[(j - 1) * NS + k]);
      } else if constexpr (LR == 2) {
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          const int k = (t + m * T) & (NS - 1);
          w[3 * m] = __ldg(&tws[k]);
          w[3 * m + 1] = __ldg(&tws[NS + k]);
          w[3 * m + 2] = __ldg(&tws[2 * NS + k]);
        }
      } else {
#pragma unroll
        for (int m = 0; m < 4; ++m) w[m] = __ldg(&tws[(t + m * T) & (NS - 1)]);
      }
    }
  }
};

// Shared scratch of a line transform: element e (logical position) of an
// array addressed by an index functor ...
template <typename E, typename Idx> struct ArrMem {
  E* sm;
  Idx idx;
  __device__ __forceinline__ void st(int e, const E& v) const { sm[idx(e)] = v; }
  __device__ __forceinline__ E ld(int e) const { return sm[idx(e)]; }
};
// ... or of three lines kept as three planes `plane` complex values apart (a
// CTrip per position, each plane addressed like one line).
template <typename R, typename Idx> struct TripMem {
  Cplx<R>* sm;
  Idx idx;
  int plane;
  __device__ __forceinline__ void st(int e, const CTrip<R>& v) const {
    const int i = idx(e);
    sm[i] = v.a;
    sm[i + plane] = v.b;
    sm[i + 2 * plane] = v.c;
  }
  __device__ __forceinline__ CTrip<R> ld(int e) const {
    const int i = idx(e);
    return CTrip<R>{sm[i], sm[i + plane], sm[i + 2 * plane]};
  }
};

// PF: twiddles a stage ahead (FP32 default: measured faster); otherwise at
// the stage itself (FP64: the extra live registers spill in the z pass).
template <int SIGN, typename R, int LGL, int LGNS, bool PF, typename E, typename Mem, typename Sync>
__device__ __forceinline__ void fft_stages_ct(E v[8], int t, const Cplx<R>* __restrict__ tw, const Mem& mem,
                                              const Sync& sync, const StageTw<R, LGL, LGNS>& cur) {
  constexpr int REM = LGL - LGNS;
  constexpr int LR = REM >= 3 ? 3 : REM;
  constexpr bool LAST = (REM == LR);
  constexpr int NS = 1 << LGNS;
  constexpr int T = 1 << (LGL - 3);
  StageTw<R, LGL, LGNS + LR> nxt;
  if constexpr (!LAST && PF) nxt.load(t, tw);
  StageTw<R, LGL, LGNS> own;
  if constexpr (!PF) own.load(t, tw);
  const StageTw<R, LGL, LGNS>& tws = PF ? cur : own;
  if constexpr (LR == 3) {
    const int k = t & (NS - 1);
    if constexpr (LGNS > 0) {
#pragma unroll
      for (int j = 1; j < 8; ++j) v[j] = twmul<SIGN>(v[j], tws.w[j - 1]);
    }
    dft8<SIGN, R>(v);
    if constexpr (!LAST) {
      const int base = ((t >> LGNS) << (LGNS + 3)) + k;
#pragma unroll
      for (int j = 0; j < 8; ++j) mem.st(base + j * NS, v[j]);
    }
  } else if constexpr (LR == 2) {
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const int b = t + m * T;
      const int k = b & (NS - 1);
      if constexpr (LGNS > 0) {
        v[m + 2] = twmul<SIGN>(v[m + 2], tws.w[3 * m]);
        v[m + 4] = twmul<SIGN>(v[m + 4], tws.w[3 * m + 1]);
        v[m + 6] = twmul<SIGN>(v[m + 6], tws.w[3 * m + 2]);
      }
      dft4<SIGN>(v[m], v[m + 2], v[m + 4], v[m + 6]);
      if constexpr (!LAST) {
        const int base = ((b >> LGNS) << (LGNS + 2)) + k;
#pragma unroll
        for (int j = 0; j < 4; ++j) mem.st(base + j * NS, v[m + 2 * j]);
      }
    }
  } else {
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const int b = t + m * T;
      const int k = b & (NS - 1);
      if constexpr (LGNS > 0) v[m + 4] = twmul<SIGN>(v[m + 4], tws.w[m]);
      dft2(v[m], v[m + 4]);
      if constexpr (!LAST) {
        const int base = ((b >> LGNS) << (LGNS + 1)) + k;
        mem.st(base, v[m]);
        mem.st(base + NS, v[m + 4]);
      }
    }
  }
  if constexpr (!LAST) {
    sync();
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = mem.ld(t + i * T);
    sync();
    fft_stages_ct<SIGN, R, LGL, LGNS + LR, PF>(v, t, tw, mem, sync, nxt);
  }
}

// Synchronisation of the threads that share one line's scratch.
struct BlockSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
// A named barrier over `count` threads (a multiple of 32: whole warps).
struct NamedSync {
  int id, count;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  }
};

// E is the element a thread holds per position: Cplx<R>, or CPair<R> for two
// adjacent columns sharing the stage's twiddles.
template <int SIGN, typename R, int LGL, typename E, typename Idx, typename Sync = BlockSync>
__device__ __forceinline__ void fft_line_ct(E v[8], int t, const Cplx<R>* __restrict__ tw, E* sm,
                                            const Idx& idx, const Sync& sync = Sync{}) {
  const StageTw<R, LGL, 0> none{};
  fft_stages_ct<SIGN, R, LGL, 0, sizeof(R) == 4>(v, t, tw, ArrMem<E, Idx>{sm, idx}, sync, none);
}
// The same with an explicit scratch policy (ArrMem, TripMem).
template <int SIGN, typename R, int LGL, bool PF = (sizeof(R) == 4), typename E, typename Mem, typename Sync>
__device__ __forceinline__ void fft_line_mem(E v[8], int t, const Cplx<R>* __restrict__ tw, const Mem& mem,
                                             const Sync& sync) {
  const StageTw<R, LGL, 0> none{};
  fft_stages_ct<SIGN, R, LGL, 0, PF>(v, t, tw, mem, sync, none);
}

// Asynchronous global -> shared copies (cp.async): B bytes (8 or 16) land at
// sdst, of which the first src_bytes are read from gsrc and the rest are
// zero-filled (src_bytes = 0 reads nothing).  Copies complete in commit
// groups; a thread sees its own copies after cp_async_wait, other threads'
// copies only after a barrier that follows their wait.
template <int B>
__device__ __forceinline__ void cp_async(void* sdst, const void* gsrc, int src_bytes) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(sdst));
  if constexpr (B == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gsrc), "r"(src_bytes)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(gsrc), "n"(B),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
// Waits until at most n of this thread's commit groups are still in flight (n <= 3).
__device__ __forceinline__ void cp_async_wait(int n) {
  switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
  }
}

// Strided shared-memory tile of a y or z pass: element e of column x of a
// [rows][2^lg] tile, with one padding row after every 8 rows.  The padding
// puts the rows that the threads of one 128-byte phase touch together in a
// Stockham stage (8 t + j, 8 (t + 1) + j, ...) into different banks.
__host__ __device__ constexpr int strided_rows(int L) { return L + (L >> 3); }
struct StridedIdxLg {
  int lg, x;
  __device__ __forceinline__ int operator()(int e) const { return ((e + (e >> 3)) << lg) + x; }
};

// Contiguous line of an x pass, XOR-swizzled within aligned groups of 16
// elements: bits 0..3 of e take bits 3..6 of e.  A bijection on each group,
// so the line needs no padding; it spreads the Stockham stage writes of a
// 128-byte phase over all banks for 8- and 16-byte elements.
__device__ __forceinline__ int swz(int e) { return e ^ ((e >> 3) & 15); }
struct SwzIdx {
  int off;
  __device__ __forceinline__ int operator()(int e) const { return off + swz(e); }
};

}  // namespace gt
