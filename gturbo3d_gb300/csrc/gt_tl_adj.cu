// C-ABI tangent-linear and adjoint RK2 step, objective and checkpointed gradient.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gt_fft.cuh"
#include "gt_handle.h"
#include "gt_internal.h"

using namespace gt;
using namespace gtc;

// ===========================================================================
// Tangent-linear and adjoint RK2 step (the differentiation extension).
// With a the stage input, bc the Coriolis source and Q(a) = P invcurl
// fft_dir(u(a) x w(a)):  nlt(a; bc) = Q(a) + P invcurl(i omega kz bc).
//   TL:  dN = P invcurl[ fft_dir(du x w + u x dw) + i omega kz dbc ]
//   adjoint (inner products of gt_adjoint.cu): with mu = invcurl P lam and
//   g = fft_inv(mu):  lam_a = curl fft_dir(w x g) + k^2 fft_dir(g x u),
//   lam_bc = -i omega kz mu.
// The RK2 step and its zeroing of the k = 0 mode (rkstep.f90:44-48,
// 100-104) are differentiated on top.
// ===========================================================================
namespace {

enum SpecOp { kOpCurl = 0, kOpK2 = 1, kOpInvcurl = 2, kOpTrunc = 3, kOpCoriolis = 4, kOpEmk = 5,
              kOpCopy = 6, kOpShell = 7, kOpZero0 = 8 };

struct F3 {
  void* p[3];
};

template <typename R>
struct AdjWork {
  gt_handle* h;
  const DevTables<R>& tb;
  std::vector<void*> blocks;
  size_t sbytes, rbytes;
  AdjWork(gt_handle* hh, const DevTables<R>& t) : h(hh), tb(t) {
    sbytes = h->g.field_elems() * sizeof(Cplx<R>);
    rbytes = (size_t)h->g.nx * h->g.ny * h->g.nz * sizeof(R);
  }
  ~AdjWork() {
    for (void* p : blocks) cudaFree(p);
  }
  int alloc(F3& f, bool real) {
    void* p = nullptr;
    const size_t b = real ? rbytes : sbytes;
    cudaError_t e = cudaMalloc(&p, 3 * b);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint workspace");
    blocks.push_back(p);
    for (int c = 0; c < 3; ++c) f.p[c] = (char*)p + c * b;
    return GT_OK;
  }
  int op(const F3& out, const F3& a, const F3* b, int o, double sgn = 1, double kmin2 = 0, double beta = 0) {
    CKI(launch_spec_op<R>(h->g, tb, out.p, a.p, b ? b->p : nullptr, o, sgn, kmin2, beta, h->stream));
    return GT_OK;
  }
  // real = C2R(spec); spec is destroyed
  int inv(const F3& real, const F3& spec) {
    for (int c = 0; c < 3; ++c)
      CKI(launch_fft_inv<R>(h->g, tb, spec.p[c], real.p[c], h->w, h->stream, hook_fn, h));
    return GT_OK;
  }
  int dir(const F3& spec, const F3& real) {
    for (int c = 0; c < 3; ++c)
      CKI(launch_fft_dir<R>(h->g, tb, real.p[c], spec.p[c], h->w, h->stream, hook_fn, h));
    return GT_OK;
  }
  int cross(const F3& out, const F3& a, const F3& b, const F3* c = nullptr, const F3* d = nullptr) {
    CKI(launch_phys_cross<R>(h->g, out.p, a.p, b.p, c ? c->p : nullptr, d ? d->p : nullptr, 1.0, 1.0,
                             h->stream));
    return GT_OK;
  }
};

// u = C2R(curl a), w = C2R(k^2 a) (tmp: one spectral group of scratch)
template <typename R>
int phys_uw(AdjWork<R>& W, const F3& a, const F3& u, const F3& w, const F3& tmp) {
  int rc;
  if ((rc = W.op(tmp, a, nullptr, kOpCurl))) return rc;
  if ((rc = W.inv(u, tmp))) return rc;
  if ((rc = W.op(tmp, a, nullptr, kOpK2))) return rc;
  return W.inv(w, tmp);
}

// dN = TL of nlt at (a; bc) in direction (da; dbc)
template <typename R>
int tl_nlt(AdjWork<R>& W, const F3& a, const F3& da, const F3& dbc, const F3& dN, const F3 s[2],
           const F3 r[5]) {
  int rc;
  if ((rc = phys_uw(W, a, r[0], r[1], s[0]))) return rc;      // u, w
  if ((rc = phys_uw(W, da, r[2], r[3], s[0]))) return rc;     // du, dw
  if ((rc = W.cross(r[4], r[2], r[1], &r[0], &r[3]))) return rc;   // du x w + u x dw
  if ((rc = W.dir(s[0], r[4]))) return rc;
  if ((rc = W.op(s[1], dbc, &s[0], kOpCoriolis, +1.0, 0, 1.0))) return rc;   // + i omega kz dbc
  if ((rc = W.op(s[0], s[1], nullptr, kOpInvcurl))) return rc;
  return W.op(dN, s[0], nullptr, kOpTrunc);
}

// (lam_a, lam_bc) += adjoint of tl_nlt at (a; bc) applied to lam
template <typename R>
int adj_nlt(AdjWork<R>& W, const F3& a, const F3& lam, const F3& lam_a, const F3& lam_bc, const F3 s[3],
            const F3 r[5]) {
  int rc;
  if ((rc = W.op(s[0], lam, nullptr, kOpTrunc))) return rc;
  if ((rc = W.op(s[1], s[0], nullptr, kOpInvcurl))) return rc;              // mu
  if ((rc = W.op(lam_bc, s[1], &lam_bc, kOpCoriolis, -1.0, 0, 1.0))) return rc;   // lam_bc += -i omega kz mu
  if ((rc = W.inv(r[4], s[1]))) return rc;                                  // g = C2R(mu)
  if ((rc = phys_uw(W, a, r[0], r[1], s[0]))) return rc;                    // u, w
  if ((rc = W.cross(r[2], r[1], r[4]))) return rc;                          // w x g
  if ((rc = W.cross(r[3], r[4], r[0]))) return rc;                          // g x u
  if ((rc = W.dir(s[0], r[2]))) return rc;
  if ((rc = W.op(s[2], s[0], &lam_a, kOpCurl, 1, 0, 1.0))) return rc;     // lam_a + curl(.)
  if ((rc = W.dir(s[0], r[3]))) return rc;
  return W.op(lam_a, s[0], &s[2], kOpK2, 1, 0, 1.0);                        // + k^2(.)
}

template <typename R>
struct StepCtx {
  AdjWork<R> W;
  F3 s[3], r[5], n1, c, t1, t2, t3;
  StepCtx(gt_handle* h, const DevTables<R>& tb) : W(h, tb) {}
  int init() {
    int rc = 0;
    for (int i = 0; i < 3 && !rc; ++i) rc = W.alloc(s[i], false);
    for (int i = 0; i < 5 && !rc; ++i) rc = W.alloc(r[i], true);
    if (!rc) rc = W.alloc(n1, false);
    if (!rc) rc = W.alloc(c, false);
    if (!rc) rc = W.alloc(t1, false);
    if (!rc) rc = W.alloc(t2, false);
    if (!rc) rc = W.alloc(t3, false);
    return rc;
  }
  // c = E(b + dt2 N1(b)), c(0) = 0, for the state b in the handle
  int stage(const F3& b) {
    gt_handle* h = W.h;
    CKI(nlt(h, b.p, b.p, n1.p, kNltOnly, 0));
    int rc;
    if ((rc = W.op(t3, b, &n1, kOpCopy, 1, 0, (double)W.tb.dt2))) return rc;
    if ((rc = W.op(c, t3, nullptr, kOpEmk))) return rc;
    return W.op(c, c, nullptr, kOpZero0);
  }
  // db' = TL of the RK2 step at b applied to db
  int tl(const F3& b, const F3& db, const F3& out) {
    int rc;
    if ((rc = stage(b))) return rc;
    if ((rc = tl_nlt(W, b, db, db, t1, s, r))) return rc;                    // dN1
    if ((rc = W.op(t2, db, &t1, kOpCopy, 1, 0, (double)W.tb.dt2))) return rc;  // db + dt2 dN1
    if ((rc = W.op(t3, t2, nullptr, kOpEmk))) return rc;
    if ((rc = W.op(t3, t3, nullptr, kOpZero0))) return rc;                   // dc
    if ((rc = tl_nlt(W, c, t3, db, t1, s, r))) return rc;                    // dN2
    if ((rc = W.op(t2, db, nullptr, kOpEmk))) return rc;                     // E db
    if ((rc = W.op(t2, t2, &t1, kOpCopy, 1, 0, (double)W.tb.dt))) return rc;  // + dt dN2
    if ((rc = W.op(out, t2, nullptr, kOpEmk))) return rc;
    return W.op(out, out, nullptr, kOpZero0);
  }
  // lam = adjoint of the RK2 step at b applied to lam' (in: lp, out: out)
  int adj(const F3& b, const F3& lp, const F3& out) {
    int rc;
    if ((rc = stage(b))) return rc;
    if ((rc = W.op(t1, lp, nullptr, kOpZero0))) return rc;                   // Z lam'
    if ((rc = W.op(t2, t1, nullptr, kOpEmk))) return rc;                     // E Z lam'
    if ((rc = W.op(out, t2, nullptr, kOpEmk))) return rc;                    // lam_b = E E Z lam'
    if ((rc = W.op(t1, t2, nullptr, kOpCopy, 1, 0, 0))) return rc;
    if ((rc = W.op(t2, t2, &t2, kOpCopy, 1, 0, (double)W.tb.dt - 1.0))) return rc;   // lam_N2 = dt E Z lam'
    // lam_c (in t3, from zero) and lam_b += lam_bc2
    if ((rc = W.op(t3, t3, nullptr, kOpCopy, 1, 0, 0))) return rc;
    CK(cudaMemsetAsync(t3.p[0], 0, W.sbytes, W.h->stream));
    CK(cudaMemsetAsync(t3.p[1], 0, W.sbytes, W.h->stream));
    CK(cudaMemsetAsync(t3.p[2], 0, W.sbytes, W.h->stream));
    if ((rc = adj_nlt(W, c, t2, t3, out, s, r))) return rc;
    if ((rc = W.op(t3, t3, nullptr, kOpZero0))) return rc;                   // Z lam_c
    if ((rc = W.op(t1, t3, nullptr, kOpEmk))) return rc;                     // E lam_c
    if ((rc = W.op(out, t1, &out, kOpCopy, 1, 0, 1.0))) return rc;           // lam_b += E lam_c
    if ((rc = W.op(t2, t1, &t1, kOpCopy, 1, 0, (double)W.tb.dt2 - 1.0))) return rc;  // lam_N1 = dt2 E lam_c
    return adj_nlt(W, b, t2, out, out, s, r);                                // lam_b += lam_a1 + lam_bc1
  }
};

template <typename R>
const DevTables<R>& tables(gt_handle* h);
template <>
const DevTables<float>& tables<float>(gt_handle* h) { return h->t32; }
template <>
const DevTables<double>& tables<double>(gt_handle* h) { return h->t64; }

template <typename R>
int tl_or_adj(gt_handle* h, const double* in[3], double* out[3], bool adjoint) {
  StepCtx<R> S(h, tables<R>(h));
  int rc = S.init();
  if (rc) return rc;
  F3 x, y, b;
  if ((rc = S.W.alloc(x, false)) || (rc = S.W.alloc(y, false))) return rc;
  for (int c = 0; c < 3; ++c) {
    if ((rc = upload_spec(h, in[c], x.p[c]))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    b.p[c] = h->b[c];
  }
  rc = adjoint ? S.adj(b, x, y) : S.tl(b, x, y);
  if (rc) return rc;
  for (int c = 0; c < 3; ++c) {
    if ((rc = download_spec(h, y.p[c], out[c]))) return rc;
    CK(cudaStreamSynchronize(h->stream));
  }
  return check_device_flag(h);
}

// J = sum over stored modes with |k| >= kmin of fac |(curl b)_k|^2
template <typename R>
int objective(gt_handle* h, StepCtx<R>& S, const F3& b, double kmin, double* J) {
  int rc;
  if ((rc = S.W.op(S.t1, b, nullptr, kOpCurl))) return rc;
  if ((rc = S.W.op(S.t1, S.t1, nullptr, kOpShell, 1, kmin * kmin))) return rc;
  const Geom& g = h->g;
  double acc = 0.0;
  std::vector<double> host((size_t)g.nz * g.ny * g.nh * 2);
  for (int c = 0; c < 3; ++c) {
    if ((rc = download_spec(h, S.t1.p[c], host.data()))) return rc;
    CK(cudaStreamSynchronize(h->stream));
    for (size_t row = 0; row < (size_t)g.nz * g.ny; ++row)
      for (int X = 0; X < g.nh; ++X) {
        const double fac = (X == 0 || X == g.nh - 1) ? 0.5 : 1.0;
        const double re = host[(row * g.nh + X) * 2], im = host[(row * g.nh + X) * 2 + 1];
        acc += fac * (re * re + im * im);
      }
  }
  *J = acc;
  return GT_OK;
}

template <typename R>
int gradient(gt_handle* h, int nsteps, int32_t seed, int K, double kmin, double* J, double* gout[3]) {
  StepCtx<R> S(h, tables<R>(h));
  int rc = S.init();
  if (rc) return rc;
  const size_t fb = S.W.sbytes;
  const int ncp = (nsteps + K - 1) / K;
  // checkpoints (state at steps 0, K, 2K, ...) and one segment of states
  std::vector<F3> cp(std::max(ncp, 1)), seg(K);
  for (auto& f : cp) if ((rc = S.W.alloc(f, false))) return rc;
  for (auto& f : seg) if ((rc = S.W.alloc(f, false))) return rc;
  F3 b0, lam, lam2, state;
  if ((rc = S.W.alloc(b0, false)) || (rc = S.W.alloc(lam, false)) || (rc = S.W.alloc(lam2, false))) return rc;
  for (int c = 0; c < 3; ++c) {
    state.p[c] = h->b[c];
    CK(cudaMemcpyAsync(b0.p[c], h->b[c], fb, cudaMemcpyDeviceToDevice, h->stream));
  }
  const bool was_in_k = h->state_in_k;
  // the forcing realisation, drawn once and replayed in every recomputation
  std::vector<ForceEntry> all;
  std::vector<size_t> offs(1, 0);
  const bool forced = h->p.forcing != GT_FORCING_NONE && !h->ht.fix.empty();
  int32_t sd = seed;
  for (int k = 0; k < nsteps; ++k) {
    if (forced) draw_forcing(h->p, h->ht, sd, all);
    offs.push_back(all.size());
  }
  auto step_k = [&](int k) {
    std::vector<ForceEntry> e(all.begin() + offs[k], all.begin() + offs[k + 1]);
    std::vector<size_t> o = {0, e.size()};
    return run_steps(h, 1, e, o);
  };
  auto copy3 = [&](const F3& dst, const F3& src) {
    for (int c = 0; c < 3; ++c)
      cudaMemcpyAsync(dst.p[c], src.p[c], fb, cudaMemcpyDeviceToDevice, h->stream);
  };
  for (int k = 0; k < nsteps; ++k) {
    if (k % K == 0) copy3(cp[k / K], state);
    if ((rc = step_k(k))) return rc;
  }
  if ((rc = objective<R>(h, S, state, kmin, J))) return rc;
  // lam = dJ/db_n = curl(1_S curl b_n)
  if ((rc = S.W.op(S.t1, state, nullptr, kOpCurl))) return rc;
  if ((rc = S.W.op(S.t1, S.t1, nullptr, kOpShell, 1, kmin * kmin))) return rc;
  if ((rc = S.W.op(lam, S.t1, nullptr, kOpCurl))) return rc;
  for (int i = ncp - 1; i >= 0; --i) {
    const int k0 = i * K, k1 = std::min(nsteps, (i + 1) * K);
    copy3(state, cp[i]);
    for (int k = k0; k < k1; ++k) {
      copy3(seg[k - k0], state);
      if (k + 1 < k1 && (rc = step_k(k))) return rc;
    }
    for (int k = k1 - 1; k >= k0; --k) {
      if ((rc = S.adj(seg[k - k0], lam, lam2))) return rc;
      copy3(lam, lam2);
    }
  }
  copy3(state, b0);
  CK(cudaStreamSynchronize(h->stream));
  h->state_in_k = was_in_k;
  for (int c = 0; c < 3; ++c) {
    if ((rc = download_spec(h, lam.p[c], gout[c]))) return rc;
    CK(cudaStreamSynchronize(h->stream));
  }
  return check_device_flag(h);
}

}  // namespace

extern "C" {

int gt_tl_step(gt_handle* h, const double* dbx, const double* dby, const double* dbz, double* ox,
               double* oy, double* oz) {
  if (!h || !dbx || !dby || !dbz || !ox || !oy || !oz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  const double* in[3] = {dbx, dby, dbz};
  double* out[3] = {ox, oy, oz};
  return h->mixed ? tl_or_adj<float>(h, in, out, false) : tl_or_adj<double>(h, in, out, false);
}

int gt_adj_step(gt_handle* h, const double* lx, const double* ly, const double* lz, double* ox,
                double* oy, double* oz) {
  if (!h || !lx || !ly || !lz || !ox || !oy || !oz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  const double* in[3] = {lx, ly, lz};
  double* out[3] = {ox, oy, oz};
  return h->mixed ? tl_or_adj<float>(h, in, out, true) : tl_or_adj<double>(h, in, out, true);
}

int gt_objective(gt_handle* h, double kmin, double* J) {
  if (!h || !J) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  F3 b;
  for (int c = 0; c < 3; ++c) b.p[c] = h->b[c];
  if (h->mixed) {
    StepCtx<float> S(h, h->t32);
    if ((rc = S.init())) return rc;
    return objective<float>(h, S, b, kmin, J);
  }
  StepCtx<double> S(h, h->t64);
  if ((rc = S.init())) return rc;
  return objective<double>(h, S, b, kmin, J);
}

int gt_gradient(gt_handle* h, int32_t nsteps, int32_t seed, int32_t checkpoint_every, double kmin,
                double* J, double* gx, double* gy, double* gz) {
  if (!h || nsteps < 1 || checkpoint_every < 1 || !J || !gx || !gy || !gz) return GT_EINVAL;
  int rc = set_dev(h);
  if (rc) return rc;
  double* out[3] = {gx, gy, gz};
  return h->mixed ? gradient<float>(h, nsteps, seed, checkpoint_every, kmin, J, out)
                  : gradient<double>(h, nsteps, seed, checkpoint_every, kmin, J, out);
}

}  // extern "C"
