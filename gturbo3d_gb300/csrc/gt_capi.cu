// C-ABI of the library: handle life cycle, state transfer, the RK2 step
// driver (the drop-in for main.f90:121-150), diagnostics, transforms and the
// initial-state / output paths.  See include/gturbo_gb.h for the contract.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gt_fft.cuh"
#include "gt_handle.h"
#include "gt_internal.h"

using namespace gt;
using namespace gtc;

namespace {

thread_local std::string g_last_error;

}  // namespace

int gtc::cuda_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return GT_ECUDA;
}

void gt::set_last_error(const std::string& msg) { g_last_error = msg; }

namespace gtc {

void hook_fn(void* ctx, int kind, bool begin) {
  gt_handle* h = static_cast<gt_handle*>(ctx);
  if (begin) ++h->launches;
  if (!h->prof) return;
  auto take = [&]() {
    cudaEvent_t e;
    if (!h->pool.empty()) {
      e = h->pool.back();
      h->pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  };
  if (begin) {
    Pending pd{kind, take(), nullptr};
    cudaEventRecord(pd.e0, h->stream);
    h->pending.push_back(pd);
  } else if (!h->pending.empty()) {
    Pending& pd = h->pending.back();
    pd.e1 = take();
    cudaEventRecord(pd.e1, h->stream);
  }
}

template <typename T> T* dptr(void* base, size_t off) {
  return reinterpret_cast<T*>(reinterpret_cast<char*>(base) + off);
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// cos and sin of 2 pi m / L: evaluated in long double on [0, pi/4] only and
// mapped to the other octants by exact symmetries, so that the table is
// exactly symmetric (W^{L/4} = -i exactly) and the same on any host.
void cos_sin(int m, int L, long double& c, long double& s) {
  if (m >= L / 2) { cos_sin(m - L / 2, L, c, s); c = -c; s = -s; return; }
  if (m > L / 4) { cos_sin(L / 2 - m, L, c, s); c = -c; return; }       // pi - phi
  if (m > L / 8) { long double c2, s2; cos_sin(L / 4 - m, L, c2, s2); c = s2; s = c2; return; }
  const long double pi = 3.141592653589793238462643383279502884L;
  const long double th = 2.0L * pi * (long double)m / (long double)L;
  c = cosl(th);
  s = sinl(th);
}

// Twiddles e^{-2 pi i m / L}, m < L.
void twiddles(int L, std::vector<double>& re, std::vector<double>& im) {
  re.assign(L, 0.0);
  im.assign(L, 0.0);
  for (int m = 0; m < L; ++m) {
    long double c, s;
    cos_sin(m, L, c, s);
    re[m] = (double)c;
    im[m] = -(double)s;
  }
}

int ilog2(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

template <typename R>
int upload_tables(gt_handle* h, DevTables<R>& t) {
  const HostTables& ht = h->ht;
  const Geom& g = h->g;
  // layout: fkx fky fkz fkxs fkys fkzs emk | xcut | twx twy twz
  const size_t nemk = ht.emk_by_k2 ? ht.emk_k2.size() : ht.emk_full.size();
  std::vector<char> buf;
  size_t off = 0;
  auto put = [&](const void* src, size_t bytes) {
    off = align_up(off, 256);
    if (buf.size() < off + bytes) buf.resize(off + bytes);
    std::memcpy(buf.data() + off, src, bytes);
    size_t at = off;
    off += bytes;
    return at;
  };
  auto putR = [&](const std::vector<double>& v) {
    std::vector<R> tmp(v.begin(), v.end());
    return put(tmp.data(), tmp.size() * sizeof(R));
  };
  const size_t o_fkx = putR(ht.fkx), o_fky = putR(ht.fky), o_fkz = putR(ht.fkz);
  const size_t o_fkxs = putR(ht.fkxs), o_fkys = putR(ht.fkys), o_fkzs = putR(ht.fkzs);
  const size_t o_emk = putR(ht.emk_by_k2 ? ht.emk_k2 : ht.emk_full);
  const size_t o_xcut = put(ht.xcut.data(), ht.xcut.size() * sizeof(int32_t));
  // Each axis: the full table tw[m] = exp(-2 pi i m / L), m < L, followed by
  // the per-stage table of the Stockham line transform (tw_stage_offset in
  // gt_fft.cuh): for every stage after the first (radix r, Ns earlier
  // points) the entries tw[j k L / (Ns r)] in [j - 1][k] order, so that the
  // lanes of a warp read consecutive entries.
  auto puttw = [&](int L) {
    std::vector<double> re, im;
    twiddles(L, re, im);
    std::vector<R> c(4 * (size_t)L, (R)0);
    for (int m = 0; m < L; ++m) {
      c[2 * m] = (R)re[m];
      c[2 * m + 1] = (R)im[m];
    }
    const int lgl = ilog2(L);
    size_t off = 0;
    for (int lgns = 0; lgns < lgl;) {
      const int lr = lgl - lgns >= 3 ? 3 : lgl - lgns;
      const int r = 1 << lr, ns = 1 << lgns;
      if (lgns > 0) {
        for (int j = 1; j < r; ++j)
          for (int k = 0; k < ns; ++k) {
            const size_t m = (size_t)j * k * (L / (ns * r));
            const size_t e = L + off + (size_t)(j - 1) * ns + k;
            c[2 * e] = (R)re[m];
            c[2 * e + 1] = (R)im[m];
          }
        off += (size_t)(r - 1) * ns;
      }
      lgns += lr;
    }
    return put(c.data(), c.size() * sizeof(R));
  };
  const size_t o_twx = puttw(g.nx), o_twy = puttw(g.ny), o_twz = puttw(g.nz);
  const size_t o_twzh = puttw(g.nz >= 2 ? g.nz / 2 : 1);
  std::vector<int32_t> tiles;
  build_ztiles(g, ht.xcut.data(), (int)sizeof(Cplx<R>), tiles);
  if (tiles.empty()) tiles = {0, 0};
  const size_t o_tiles = put(tiles.data(), tiles.size() * sizeof(int32_t));
  size_t o_tl[11], o_tlzc[11];
  int n_tl[11];
  for (int lg = 0; lg < 11; ++lg) {
    std::vector<int32_t> tl;
    build_ztiles(g, ht.xcut.data(), (int)sizeof(Cplx<R>), tl, 1 << lg);
    if (tl.empty()) tl = {0, 0};
    o_tl[lg] = put(tl.data(), tl.size() * sizeof(int32_t));
    n_tl[lg] = (int)(tl.size() / 2);
    // kept half range of each tile's first column: xcut[z][y] is non-increasing in |kz|
    std::vector<int32_t> zc(tl.size() / 2, 0);
    for (size_t e = 0; e < zc.size(); ++e) {
      const int X = tl[2 * e] << lg, y = tl[2 * e + 1];
      int z = 0;
      while (z + 1 <= g.nz / 2 && ht.xcut[(size_t)(z + 1) * g.ny + y] > X) ++z;
      zc[e] = z;
    }
    if (zc.empty()) zc = {0};
    o_tlzc[lg] = put(zc.data(), zc.size() * sizeof(int32_t));
  }
  (void)nemk;
  void* mem = nullptr;
  CK(cudaMalloc(&mem, buf.size()));
  CK(cudaMemcpy(mem, buf.data(), buf.size(), cudaMemcpyHostToDevice));
  h->tab_mem = mem;
  t.fkx = dptr<const R>(mem, o_fkx);
  t.fky = dptr<const R>(mem, o_fky);
  t.fkz = dptr<const R>(mem, o_fkz);
  t.fkxs = dptr<const R>(mem, o_fkxs);
  t.fkys = dptr<const R>(mem, o_fkys);
  t.fkzs = dptr<const R>(mem, o_fkzs);
  t.emk = dptr<const R>(mem, o_emk);
  t.emk_by_k2 = ht.emk_by_k2 ? 1 : 0;
  t.xcut = dptr<const int32_t>(mem, o_xcut);
  t.twx = dptr<const void>(mem, o_twx);
  t.twy = dptr<const void>(mem, o_twy);
  t.twz = dptr<const void>(mem, o_twz);
  t.twzh = dptr<const void>(mem, o_twzh);
  t.omega = (R)h->p.omega;
  t.dt = (R)h->p.dt;
  t.dt2 = (R)(h->p.dt2_mode == GT_DT2_RK2 ? 0.5 * h->p.dt : 0.0);
  t.scale = (R)(1.0 / ((double)g.nx * g.ny * g.nz));
  t.truncate = h->p.truncate;
  t.ztiles = dptr<const int32_t>(mem, o_tiles);
  t.nztiles = (int)(tiles.size() / 2);
  for (int lg = 0; lg < 11; ++lg) {
    t.ztl[lg] = dptr<const int32_t>(mem, o_tl[lg]);
    t.nztl[lg] = n_tl[lg];
    t.ztlzc[lg] = dptr<const int32_t>(mem, o_tlzc[lg]);
  }
  t.xa = ht.xcut[0];
  return GT_OK;
}

void free_handle(gt_handle* h) {
  if (!h) return;
  cudaSetDevice(h->p.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& pd : h->pending) {
    if (pd.e0) cudaEventDestroy(pd.e0);
    if (pd.e1) cudaEventDestroy(pd.e1);
  }
  for (auto e : h->pool) cudaEventDestroy(e);
  for (int i = 0; i < 2; ++i) {
    if (h->d_force[i]) cudaFree(h->d_force[i]);
    if (h->h_force[i]) cudaFreeHost(h->h_force[i]);
    if (h->force_copied[i]) cudaEventDestroy(h->force_copied[i]);
  }
  if (h->fields_mem && h->owns_fields) cudaFree(h->fields_mem);
  if (h->stage) cudaFree(h->stage);
  if (h->tab_mem) cudaFree(h->tab_mem);
  if (h->d_partials) cudaFree(h->d_partials);
  if (h->d_result) cudaFree(h->d_result);
  if (h->d_count) cudaFree(h->d_count);
  if (h->d_err) cudaFree(h->d_err);
  if (h->h_result) cudaFreeHost(h->h_result);
  if (h->h_flag) cudaFreeHost(h->h_flag);
  if (h->pm.stream2) {
    cudaStreamSynchronize((cudaStream_t)h->pm.stream2);
    cudaStreamDestroy((cudaStream_t)h->pm.stream2);
  }
  if (h->pm.ev_fork) cudaEventDestroy((cudaEvent_t)h->pm.ev_fork);
  if (h->pm.ev_join) cudaEventDestroy((cudaEvent_t)h->pm.ev_join);
  if (h->pm.ev_mid) cudaEventDestroy((cudaEvent_t)h->pm.ev_mid);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// ---- dispatch on precision ----------------------------------------------
int nlt(gt_handle* h, void* const a[3], void* const bcor[3], void* const out[3], int mode,
        int pruned) {
  const PassTuning& pm = h->pm;
  if (h->mixed)
    return launch_nlt<float>(h->g, h->t32, a, bcor, out, h->w, mode, pruned, &pm, h->d_err, h->stream,
                             hook_fn, h);
  return launch_nlt<double>(h->g, h->t64, a, bcor, out, h->w, mode, pruned, &pm, h->d_err, h->stream,
                            hook_fn, h);
}

// Both nonlinear terms of one RK2 step, b -> c -> b (main.f90:124-146).
int rk2_nlts(gt_handle* h, int pruned) {
  const PassTuning& pm = h->pm;
  if (h->mixed)
    return launch_rk2_nlts<float>(h->g, h->t32, h->b, h->c, h->w, pruned, &pm, h->d_err, h->stream,
                                  hook_fn, h);
  return launch_rk2_nlts<double>(h->g, h->t64, h->b, h->c, h->w, pruned, &pm, h->d_err, h->stream,
                                 hook_fn, h);
}

// Reads (and clears) the device error flag of the bounded waits.
int check_device_flag(gt_handle* h) {
  CK(cudaMemcpyAsync(h->h_flag, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return take_device_flag(h);
}

int take_device_flag(gt_handle* h) {
  const int v = *h->h_flag;
  if (v) {
    CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    g_last_error = "a bounded device wait timed out";
    return v;
  }
  return GT_OK;
}

bool use_pruning(const gt_handle* h) {
  return h->prune_enabled && h->p.truncate == 1 && h->state_in_k && h->forcing_in_k;
}

bool mode_in_k(const gt_handle* h, int z, int y, int x) {
  return x < h->ht.xcut[(size_t)z * h->g.ny + y];
}

// Recomputes whether the device state is zero outside K.
int refresh_state_in_k(gt_handle* h) {
  int rc = h->mixed ? launch_count_outside<float>(h->g, h->t32, h->b, h->d_count, h->stream)
                    : launch_count_outside<double>(h->g, h->t64, h->b, h->d_count, h->stream);
  if (rc) return cuda_fail((cudaError_t)rc, "launch_count_outside");
  unsigned long long n = 1;
  CK(cudaMemcpyAsync(&n, h->d_count, sizeof(n), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->state_in_k = (n == 0);
  return GT_OK;
}

int force(gt_handle* h, const ForceEntry* d, int n, int serial) {
  if (h->mixed) return launch_force<float>(h->g, h->b, d, n, serial, h->stream, hook_fn, h);
  return launch_force<double>(h->g, h->b, d, n, serial, h->stream, hook_fn, h);
}

// FP64 staging [n complex] <-> working precision
int to_working(gt_handle* h, const void* stage, void* dst, size_t n) {
  Geom g1 = h->g;
  g1.nz = 1; g1.ny = 1; g1.nhp = (int)n;   // field_elems() == n
  if (h->mixed) return launch_convert<float>(g1, stage, dst, 1, h->stream, hook_fn, h);
  CK(cudaMemcpyAsync(dst, stage, n * 16, cudaMemcpyDeviceToDevice, h->stream));
  return 0;
}

int from_working(gt_handle* h, const void* src, void* stage, size_t n) {
  Geom g1 = h->g;
  g1.nz = 1; g1.ny = 1; g1.nhp = (int)n;
  if (h->mixed) return launch_convert<float>(g1, src, stage, 0, h->stream, hook_fn, h);
  CK(cudaMemcpyAsync(stage, src, n * 16, cudaMemcpyDeviceToDevice, h->stream));
  return 0;
}

int upload_spec(gt_handle* h, const double* host, void* dst) {
  const Geom& g = h->g;
  CK(cudaMemcpy2DAsync(h->stage, (size_t)g.nhp * 16, host, (size_t)g.nh * 16, (size_t)g.nh * 16,
                       (size_t)g.ny * g.nz, cudaMemcpyHostToDevice, h->stream));
  CKI(to_working(h, h->stage, dst, g.field_elems()));
  return GT_OK;
}

int download_spec(gt_handle* h, const void* src, double* host) {
  const Geom& g = h->g;
  CKI(from_working(h, src, h->stage, g.field_elems()));
  CK(cudaMemcpy2DAsync(host, (size_t)g.nh * 16, h->stage, (size_t)g.nhp * 16, (size_t)g.nh * 16,
                       (size_t)g.ny * g.nz, cudaMemcpyDeviceToHost, h->stream));
  return GT_OK;
}

int upload_real(gt_handle* h, const double* host, void* dst) {
  const Geom& g = h->g;
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  CK(cudaMemcpyAsync(h->stage, host, n * 8, cudaMemcpyHostToDevice, h->stream));
  CKI(to_working(h, h->stage, dst, n / 2));
  return GT_OK;
}

int download_real(gt_handle* h, const void* src, double* host) {
  const Geom& g = h->g;
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  CKI(from_working(h, src, h->stage, n / 2));
  CK(cudaMemcpyAsync(host, h->stage, n * 8, cudaMemcpyDeviceToHost, h->stream));
  return GT_OK;
}

int fft_inv_dev(gt_handle* h, void* spec, void* real) {
  if (h->mixed) return launch_fft_inv<float>(h->g, h->t32, spec, real, h->w, h->stream, hook_fn, h);
  return launch_fft_inv<double>(h->g, h->t64, spec, real, h->w, h->stream, hook_fn, h);
}

int fft_dir_dev(gt_handle* h, const void* real, void* spec) {
  if (h->mixed) return launch_fft_dir<float>(h->g, h->t32, real, spec, h->w, h->stream, hook_fn, h);
  return launch_fft_dir<double>(h->g, h->t64, real, spec, h->w, h->stream, hook_fn, h);
}

int point(gt_handle* h, void* const a[3], int op, double* partial, int npartial) {
  if (h->mixed)
    return launch_point<float>(h->g, h->t32, a, op, partial, npartial, h->stream, hook_fn, h);
  return launch_point<double>(h->g, h->t64, a, op, partial, npartial, h->stream, hook_fn, h);
}

int copy_fields(gt_handle* h, void* const dst[3], void* const src[3]) {
  const size_t bytes = h->g.field_elems() * h->csize;
  for (int c = 0; c < 3; ++c)
    CK(cudaMemcpyAsync(dst[c], src[c], bytes, cudaMemcpyDeviceToDevice, h->stream));
  return GT_OK;
}

int ensure_force_cap(gt_handle* h, int slot, size_t n) {
  if (h->force_cap[slot] >= n) return GT_OK;
  size_t cap = 256;
  while (cap < n) cap *= 2;
  CK(cudaStreamSynchronize(h->stream));
  if (h->d_force[slot]) cudaFree(h->d_force[slot]);
  if (h->h_force[slot]) cudaFreeHost(h->h_force[slot]);
  h->d_force[slot] = nullptr;
  h->h_force[slot] = nullptr;
  h->force_cap[slot] = 0;
  CK(cudaMalloc(&h->d_force[slot], cap * sizeof(ForceEntry)));
  CK(cudaMallocHost(&h->h_force[slot], cap * sizeof(ForceEntry)));
  h->force_cap[slot] = cap;
  return GT_OK;
}

// Enqueues nsteps RK2 steps; entries[s] are the forcing adds of step s.
int run_steps(gt_handle* h, int nsteps, const std::vector<ForceEntry>& all,
              const std::vector<size_t>& offs) {
  const int slot = h->force_slot;
  h->force_slot ^= 1;
  const ForceEntry* dent = nullptr;
  if (!all.empty()) {
    int rc = ensure_force_cap(h, slot, all.size());
    if (rc) return rc;
    CK(cudaEventSynchronize(h->force_copied[slot]));   // previous user of this slot is done
    std::memcpy(h->h_force[slot], all.data(), all.size() * sizeof(ForceEntry));
    CK(cudaMemcpyAsync(h->d_force[slot], h->h_force[slot], all.size() * sizeof(ForceEntry),
                       cudaMemcpyHostToDevice, h->stream));
    CK(cudaEventRecord(h->force_copied[slot], h->stream));
    dent = h->d_force[slot];
  }
  const int pr = use_pruning(h) ? 1 : 0;
  for (int s = 0; s < nsteps; ++s) {
    CKI(rk2_nlts(h, pr));                      // main.f90:124-146
    if (dent) {                               // main.f90:149
      const size_t n = offs[s + 1] - offs[s];
      const bool serial = !entries_unique(all.data() + offs[s], n);
      CKI(force(h, dent + offs[s], (int)n, serial ? 1 : 0));
    }
  }
  return GT_OK;
}

int set_dev(gt_handle* h) {
  CK(cudaSetDevice(h->p.device));
  const cudaError_t stale = cudaGetLastError();   // a non-sticky error of an earlier call
  if (stale != cudaSuccess) g_last_error = std::string("cleared earlier error: ") + cudaGetErrorString(stale);
  return GT_OK;
}

}  // namespace gtc

// A handle; with ext_fields its twelve fields live in memory the caller
// owns (an ensemble class slab) and are not freed with the handle.
int gtc::create_handle(const gt_params* p, gt_handle** out, void* ext_fields) {
  if (!p || !out) return GT_EINVAL;
  *out = nullptr;
  int rc = gt_params_validate(p);
  if (rc) return rc;
  gt_handle* h = new (std::nothrow) gt_handle();
  if (!h) return GT_ENOMEM;
  h->p = *p;
  rc = build_tables(*p, h->ht);
  if (rc) { delete h; return rc; }
  h->mixed = p->precision == GT_PREC_MIXED;
  h->csize = h->mixed ? 8 : 16;
  Geom& g = h->g;
  g.nx = p->nx; g.ny = p->ny; g.nz = p->nz;
  g.nh = p->nx / 2 + 1;
  const int align = 128 / h->csize;
  g.nhp = (g.nh + align - 1) / align * align;
  g.lnx = ilog2(g.nx); g.lny = ilog2(g.ny); g.lnz = ilog2(g.nz);
  size_t need = 0;
  gt_memory_estimate(p, &need);
  uint64_t budget = 0;
  gt_get_memory_budget(&budget);
  if (budget > 0 && need > budget) {   // decided on the host, before any CUDA call
    g_last_error = "grid needs " + std::to_string(need) + " device bytes, over the budget of " +
                   std::to_string(budget) + " set by gt_set_memory_budget";
    delete h;
    return GT_ENOMEM;
  }
  cudaError_t e = cudaSetDevice(p->device);
  if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaSetDevice"); }
  size_t freeb = 0, totalb = 0;
  e = cudaMemGetInfo(&freeb, &totalb);
  if (e != cudaSuccess) { delete h; return cuda_fail(e, "cudaMemGetInfo"); }
  if (need + ((size_t)1 << 28) > freeb) {
    g_last_error = "grid needs more device memory than is free";
    delete h;
    return GT_ENOMEM;
  }
#define CKH(call)                                    \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) {                         \
      int r_ = cuda_fail(e_, #call);                 \
      free_handle(h);                                \
      return e_ == cudaErrorMemoryAllocation ? GT_ENOMEM : r_; \
    }                                                \
  } while (0)
  CKH(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  {
    // second stream and fork / join events for the overlap of the z inverse
    // pass's k^2 half with the curl half
    cudaStream_t s2 = nullptr;
    cudaEvent_t ef = nullptr, ej = nullptr;
    CKH(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
    h->pm.stream2 = s2;
    CKH(cudaEventCreateWithFlags(&ef, cudaEventDisableTiming));
    h->pm.ev_fork = ef;
    CKH(cudaEventCreateWithFlags(&ej, cudaEventDisableTiming));
    h->pm.ev_join = ej;
    cudaEvent_t em = nullptr;
    CKH(cudaEventCreateWithFlags(&em, cudaEventDisableTiming));
    h->pm.ev_mid = em;
  }
  const size_t fbytes = g.field_elems() * h->csize;
  if (ext_fields) {
    h->fields_mem = ext_fields;
    h->owns_fields = false;
  } else {
    CKH(cudaMalloc(&h->fields_mem, 12 * fbytes));
  }
  CKH(cudaMemsetAsync(h->fields_mem, 0, 12 * fbytes, h->stream));
  for (int c = 0; c < 3; ++c) {
    h->b[c] = dptr<void>(h->fields_mem, c * fbytes);
    h->c[c] = dptr<void>(h->fields_mem, (3 + c) * fbytes);
  }
  for (int c = 0; c < 6; ++c) h->w[c] = dptr<void>(h->fields_mem, (6 + c) * fbytes);
  CKH(cudaMalloc(&h->stage, g.field_elems() * 16));
  rc = h->mixed ? upload_tables<float>(h, h->t32) : upload_tables<double>(h, h->t64);
  if (rc) { free_handle(h); return rc; }
  const int nbin = g.nx / 2;
  h->nresult = kDiagScalars + 3 * nbin;
  const int nblk = diag_blocks(g);
  h->npartials = std::max(nblk * h->nresult, 65536);
  CKH(cudaMalloc(&h->d_partials, (size_t)(h->npartials + 1) * sizeof(double)));
  CKH(cudaMalloc(&h->d_result, (size_t)h->nresult * sizeof(double)));
  CKH(cudaMallocHost(&h->h_result, (size_t)h->nresult * sizeof(double)));
  CKH(cudaMallocHost(&h->h_flag, sizeof(int)));
  for (int i = 0; i < 2; ++i) CKH(cudaEventCreateWithFlags(&h->force_copied[i], cudaEventDisableTiming));
  CKH(cudaMalloc(&h->d_count, sizeof(unsigned long long)));
  CKH(cudaMalloc(&h->d_err, sizeof(int)));
  CKH(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
  // default x pass per grid: the parking variant where it measured faster
  // (FP32, NX = 512: 1.09 against 1.12 ms); at NX = 256 and 1024 and in FP64
  // the register-resident one
  h->pm.x_fused = (h->mixed && g.lnx == 9) ? 3 : 2;
  // z forward pass on cluster pairs for mixed z columns of 1024+ points (4.68 -> 4.31 ms at 1024^3);
  // TMA-loaded tiles for mixed z columns of 256 and 512 points: the z forward pass (0.435 -> 0.356 ms
  // at 512^3, 0.061 -> 0.055 ms at 256^3) and the z inverse pass (0.549 -> 0.512, 0.075 -> 0.070 ms)
  h->pm.z_cluster = (h->mixed && g.lnz >= 10) ? 1 : 0;
  // the z inverse pass's tensor stores (bit 4) only at 256 points: 0.0710 -> 0.0671 ms at 256^3,
  // but 0.513 -> 0.518 ms at 512^3
  h->pm.z_tma = h->mixed ? (g.lnz == 8 ? 7 : (g.lnz == 9 ? 3 : 0)) : 0;
  h->state_in_k = true;   // the zero state
  h->forcing_in_k = true;
  for (size_t m = 0; m < h->ht.fix.size(); ++m) {
    const int x = h->ht.fix[m], y = h->ht.fiy[m], z = h->ht.fiz[m];
    if (!mode_in_k(h, z, y, x) || !mode_in_k(h, h->ht.kc[z], h->ht.jc[y], x)) h->forcing_in_k = false;
  }
  CKH(cudaStreamSynchronize(h->stream));
#undef CKH
  *out = h;
  return GT_OK;
}

extern "C" {

int gt_create(const gt_params* p, gt_handle** out) { return create_handle(p, out, nullptr); }

int gt_destroy(gt_handle* h) {
  if (!h) return GT_EINVAL;
  free_handle(h);
  return GT_OK;
}

int gt_set_state(gt_handle* h, const double* bx, const double* by, const double* bz) {
  if (!h || !bx || !by || !bz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  const double* src[3] = {bx, by, bz};
  for (int c = 0; c < 3; ++c)
    if ((rc = upload_spec(h, src[c], h->b[c]))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return refresh_state_in_k(h);
}

int gt_get_state(gt_handle* h, double* bx, double* by, double* bz) {
  if (!h || !bx || !by || !bz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  double* dst[3] = {bx, by, bz};
  for (int c = 0; c < 3; ++c) {
    if ((rc = download_spec(h, h->b[c], dst[c]))) return rc;
    CK(cudaStreamSynchronize(h->stream));   // the staging buffer is reused
  }
  return check_device_flag(h);
}

int gt_rk2_step(gt_handle* h, int32_t nsteps, int32_t* seed_inout) {
  if (!h || nsteps < 0) return GT_EINVAL;
  const bool forced = h->p.forcing != GT_FORCING_NONE && !h->ht.fix.empty();
  if (forced && !seed_inout) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  std::vector<ForceEntry> all;
  std::vector<size_t> offs(1, 0);
  int32_t seed = seed_inout ? *seed_inout : 0;
  for (int s = 0; s < nsteps; ++s) {
    if (forced) draw_forcing(h->p, h->ht, seed, all);
    offs.push_back(all.size());
  }
  rc = run_steps(h, nsteps, all, offs);
  if (rc) return rc;
  CK(cudaGetLastError());
  if (seed_inout) *seed_inout = seed;
  return GT_OK;
}

int gt_rk2_step_coeffs(gt_handle* h, int32_t n, const int32_t* ix, const int32_t* iy,
                       const int32_t* iz, const double* dF) {
  if (!h || n < 0 || (n > 0 && (!ix || !iy || !iz || !dF))) return GT_EINVAL;
  const Geom& g = h->g;
  std::vector<ForceEntry> all;
  for (int e = 0; e < n; ++e) {
    if (ix[e] < 0 || ix[e] >= g.nh || iy[e] < 0 || iy[e] >= g.ny || iz[e] < 0 || iz[e] >= g.nz)
      return GT_EINVAL;
    ForceEntry en{iz[e], iy[e], ix[e], 7, {}};
    for (int q = 0; q < 6; ++q) en.inc[q] = dF[(size_t)e * 6 + q];
    all.push_back(en);
  }
  int rc = set_dev(h);
  if (rc) return rc;
  std::vector<size_t> offs = {0, all.size()};
  rc = run_steps(h, 1, all, offs);
  for (const ForceEntry& en : all)
    if (!mode_in_k(h, en.z, en.y, en.x)) h->state_in_k = false;
  return rc;
}

int gt_nonlinear(gt_handle* h, const double* ax, const double* ay, const double* az,
                 double* nx_out, double* ny_out, double* nz_out) {
  if (!h || !ax || !ay || !az || !nx_out || !ny_out || !nz_out) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  const double* src[3] = {ax, ay, az};
  for (int c = 0; c < 3; ++c)
    if ((rc = upload_spec(h, src[c], h->c[c]))) return rc;
  CKI(nlt(h, h->c, h->b, h->c, kNltOnly));
  double* dst[3] = {nx_out, ny_out, nz_out};
  for (int c = 0; c < 3; ++c) {
    if ((rc = download_spec(h, h->c[c], dst[c]))) return rc;
    CK(cudaStreamSynchronize(h->stream));
  }
  return GT_OK;
}

int gt_diagnostics(gt_handle* h, gt_diag* out, double* ek, double* ek2d, double* flux) {
  if (!h || !out) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  const Geom& g = h->g;
  if (flux) CKI(nlt(h, h->b, h->b, h->c, kNltOnly));   // N1 = nlt(b) (main.f90:131-136)
  const int nblk = diag_blocks(g);
  if (h->mixed)
    CKI(launch_diag<float>(g, h->t32, h->b, flux ? h->c : nullptr, h->p.nu, h->p.alpnu, h->p.mu,
                           h->p.alpmu, h->d_partials, nblk, h->d_result, h->stream, hook_fn, h));
  else
    CKI(launch_diag<double>(g, h->t64, h->b, flux ? h->c : nullptr, h->p.nu, h->p.alpnu, h->p.mu,
                            h->p.alpmu, h->d_partials, nblk, h->d_result, h->stream, hook_fn, h));
  CK(cudaMemcpyAsync(h->h_result, h->d_result, (size_t)h->nresult * sizeof(double),
                     cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  const double* r = h->h_result;
  for (int q = 0; q < 9; ++q) {
    out->energy[q] = r[q];
    out->enstrophy[q] = r[9 + q];
  }
  out->helicity = r[18];
  out->nonfinite = (int64_t)r[19];
  out->inpe = h->ht.inpe;
  out->inpz = h->ht.inpz;
  const int nbin = g.nx / 2;
  const double* sp = r + kDiagScalars;
  if (ek) for (int s = 0; s < nbin; ++s) ek[s] = sp[s];
  if (ek2d) for (int s = 0; s < nbin; ++s) ek2d[s] = sp[nbin + s];
  if (flux) {
    // diagnostics.f90:88-90: spf(i) = sum(sp(i:NBIN)); slot ib holds shell int|k| = ib
    const double* fl = sp + 2 * nbin;
    for (int s = 0; s < nbin; ++s) {
      double acc = 0.0;
      for (int ib = s + 1; ib < nbin; ++ib) acc += fl[ib];
      flux[s] = acc;
    }
  }
  return GT_OK;
}

int gt_energy(gt_handle* h, double* energy_xyz) {
  if (!h || !energy_xyz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  const int nblk = h->npartials / 3;          // the reduction's block count is capped by the partials
  const int pr = use_pruning(h) ? 1 : 0;   // state zero outside the kept set
  if (h->mixed)
    CKI(launch_energy<float>(h->g, h->t32, h->b, pr, h->d_partials, nblk, h->d_result, h->stream,
                             hook_fn, h));
  else
    CKI(launch_energy<double>(h->g, h->t64, h->b, pr, h->d_partials, nblk, h->d_result, h->stream,
                              hook_fn, h));
  CK(cudaMemcpyAsync(h->h_result, h->d_result, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                     h->stream));
  // the device error flag comes back with the result, under the same synchronisation
  CK(cudaMemcpyAsync(h->h_flag, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int c = 0; c < 3; ++c) energy_xyz[c] = h->h_result[c];
  return take_device_flag(h);
}

int gt_fft_dir(gt_handle* h, const double* real_in, double* spec_out) {
  if (!h || !real_in || !spec_out) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  if ((rc = upload_real(h, real_in, h->w[1]))) return rc;
  CKI(fft_dir_dev(h, h->w[1], h->w[0]));
  if ((rc = download_spec(h, h->w[0], spec_out))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return GT_OK;
}

int gt_fft_inv(gt_handle* h, const double* spec_in, double* real_out) {
  if (!h || !spec_in || !real_out) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  if ((rc = upload_spec(h, spec_in, h->w[0]))) return rc;
  CKI(fft_inv_dev(h, h->w[0], h->w[1]));
  if ((rc = download_real(h, h->w[1], real_out))) return rc;
  CK(cudaStreamSynchronize(h->stream));
  return GT_OK;
}

int gt_velocity(gt_handle* h, double* ux, double* uy, double* uz) {
  if (!h || !ux || !uy || !uz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  void* const u[3] = {h->w[3], h->w[4], h->w[5]};
  if ((rc = copy_fields(h, u, h->b))) return rc;
  CKI(point(h, u, 0, nullptr, 0));                        // curl (main.f90:195)
  double* dst[3] = {ux, uy, uz};
  for (int c = 0; c < 3; ++c) {                           // fft_inv x3 (main.f90:197-199)
    CKI(fft_inv_dev(h, u[c], h->w[0]));
    if ((rc = download_real(h, h->w[0], dst[c]))) return rc;
    CK(cudaStreamSynchronize(h->stream));
  }
  return GT_OK;
}

int gt_set_state_physical(gt_handle* h, const double* ux, const double* uy, const double* uz,
                          double* cc) {
  if (!h || !ux || !uy || !uz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  void* const a[3] = {h->w[3], h->w[4], h->w[5]};
  const double* src[3] = {ux, uy, uz};
  for (int c = 0; c < 3; ++c) {                           // fft_dir x3 (main.f90:91-93)
    if ((rc = upload_real(h, src[c], h->w[0]))) return rc;
    CKI(fft_dir_dev(h, h->w[0], a[c]));
    CK(cudaStreamSynchronize(h->stream));                 // staging reuse
  }
  CKI(point(h, a, 3, h->d_partials, h->npartials));       // incompr (main.f90:96)
  CKI(point(h, a, 1, nullptr, 0));                        // invcurl (main.f90:99)
  if (h->p.truncate == 1) CKI(point(h, a, 2, nullptr, 0));  // trunc x3 (main.f90:102-106)
  if ((rc = copy_fields(h, h->b, a))) return rc;
  double ccv = 0.0;
  CK(cudaMemcpyAsync(&ccv, h->d_partials + h->npartials, sizeof(double), cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (cc) *cc = ccv;
  return refresh_state_in_k(h);
}

int gt_check_finite(gt_handle* h) {
  if (!h) return GT_EINVAL;
  gt_diag d;
  int rc = gt_diagnostics(h, &d, nullptr, nullptr, nullptr);
  if (rc) return rc;
  return d.nonfinite ? GT_ENONFINITE : GT_OK;
}

int gt_set_tuning(gt_handle* h, const char* key, int32_t value) {
  if (!h || !key) return GT_EINVAL;
  const std::string k(key);
  if (k == "y_tx" && (value == 0 || value == 2 || value == 4 || value == 8 || value == 16)) h->pm.y_tx = value;
  else if (k == "z_tx" && (value == 0 || value == 2 || value == 4 || value == 8 || value == 16)) h->pm.z_tx = value;
  else if (k == "x_fused" && value >= 0 && value <= 3) h->pm.x_fused = value;
  else if (k == "y_pairs") h->pm.y_pairs = value != 0;
  else if (k == "y_prefetch" && value >= 0 && value <= 2) h->pm.y_prefetch = value;
  else if (k == "overlap") h->pm.overlap = value != 0;
  else if (k == "slab_pipe") h->pm.slab_pipe = value != 0;
  else if (k == "zf_pipe") h->pm.zf_pipe = value != 0;
  else if (k == "z_cluster" && value >= 0 && value <= 1) h->pm.z_cluster = value;
  else if (k == "z_tma" && value >= 0 && value <= 7) h->pm.z_tma = value;
  else if (k == "fuse_stage") h->pm.fuse_stage = value != 0;
  else if (k == "z_split" && value >= 0 && value <= 3) h->pm.z_split = value;
  else return GT_EINVAL;
  return GT_OK;
}

int gt_get_tuning(gt_handle* h, const char* key, int32_t* value) {
  if (!h || !key || !value) return GT_EINVAL;
  const std::string k(key);
  if (k == "y_tx") *value = h->pm.y_tx;
  else if (k == "z_tx") *value = h->pm.z_tx;
  else if (k == "x_fused") *value = h->pm.x_fused;
  else if (k == "y_pairs") *value = h->pm.y_pairs;
  else if (k == "y_prefetch") *value = h->pm.y_prefetch;
  else if (k == "overlap") *value = h->pm.overlap;
  else if (k == "slab_pipe") *value = h->pm.slab_pipe;
  else if (k == "zf_pipe") *value = h->pm.zf_pipe;
  else if (k == "z_cluster") *value = h->pm.z_cluster;
  else if (k == "z_tma") *value = h->pm.z_tma;
  else if (k == "fuse_stage") *value = h->pm.fuse_stage;
  else if (k == "z_split") *value = h->pm.z_split;
  else return GT_EINVAL;
  return GT_OK;
}

int gt_selftest_wait_timeout(gt_handle* h) {
  if (!h) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  if ((rc = launch_wait_selftest(h->d_err, h->stream))) return cuda_fail((cudaError_t)rc, "launch_wait_selftest");
  return check_device_flag(h);
}

int gt_set_pruning(gt_handle* h, int32_t enable) {
  if (!h) return GT_EINVAL;
  h->prune_enabled = enable != 0;
  return GT_OK;
}

int gt_pruning_active(gt_handle* h, int32_t* active) {
  if (!h || !active) return GT_EINVAL;
  *active = use_pruning(h) ? 1 : 0;
  return GT_OK;
}

int gt_get_stream(gt_handle* h, void** stream) {
  if (!h || !stream) return GT_EINVAL;
  *stream = (void*)h->stream;
  return GT_OK;
}

int gt_launch_count(gt_handle* h, int64_t* count) {
  if (!h || !count) return GT_EINVAL;
  *count = h->launches;
  return GT_OK;
}

int gt_profile_enable(gt_handle* h, int32_t on) {
  if (!h) return GT_EINVAL;
  h->prof = on != 0;
  return GT_OK;
}

int gt_profile_read(gt_handle* h, int32_t cap, char* names, int64_t* launches, double* ms,
                    int32_t* nkinds) {
  if (!h || cap < 0) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->stream));
  for (auto& pd : h->pending) {
    if (pd.e1) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, pd.e0, pd.e1) == cudaSuccess) {
        h->kind_ms[pd.kind] += t;
        h->kind_launches[pd.kind] += 1;
      }
      h->pool.push_back(pd.e1);
    }
    h->pool.push_back(pd.e0);
  }
  h->pending.clear();
  int n = 0;
  for (int k = 0; k < kNumKinds && n < cap; ++k) {
    if (h->kind_launches[k] == 0) continue;
    if (names) {
      std::strncpy(names + 32 * n, kernel_kind_name(k), 31);
      names[32 * n + 31] = '\0';
    }
    if (launches) launches[n] = h->kind_launches[k];
    if (ms) ms[n] = h->kind_ms[k];
    ++n;
  }
  for (int k = 0; k < kNumKinds; ++k) {
    h->kind_launches[k] = 0;
    h->kind_ms[k] = 0.0;
  }
  if (nkinds) *nkinds = n;
  return GT_OK;
}

const char* gt_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
