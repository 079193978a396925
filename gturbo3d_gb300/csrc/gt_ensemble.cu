// C-ABI batched ensemble runner.
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
// Ensemble: independent members of possibly different grids and parameters,
// advanced together.  Members of one grid class (same grid, box, precision
// and truncation; two or more members) share one device slab for their
// fields, so that every pass of the RK2 step runs as ONE launch for the whole
// class (the member index is a spare grid axis, Batch<R>), with each member's
// own integrating factor, Omega, dt and forcing.  Classes run concurrently on
// their own streams; members of no class run on their own streams.  In graph
// mode one captured CUDA graph advances every member by a chunk of 64 steps;
// the forcing is drawn on the host per chunk and read on the device by step
// index.
// ===========================================================================
namespace {

constexpr int kEnsembleChunk = 64;

// One grid class launched as one batch.
struct EnsClass {
  std::vector<int> members;     // ensemble indices; member k's fields are slab part k
  void* slab = nullptr;         // members x 12 fields
  void* btab = nullptr;         // members' emk tables, then their (omega, dt, dt2)
  int emk_len = 0;
  size_t scal_off = 0;          // byte offset of the scalars in btab
  cudaStream_t stream = nullptr;
  cudaEvent_t join = nullptr;
  // forcing of a chunk: entries [member][step][nmax], counts per member
  ForceEntry* d_ent = nullptr;
  int* d_count = nullptr;
  int nmax = 0;
  int* d_step = nullptr;
};

}  // namespace

struct gt_ensemble {
  std::vector<gt_handle*> m;
  std::vector<int> cls_of;      // class index of each member, -1 if it runs alone
  std::vector<EnsClass> cls;
  bool batching = true;
  int device = 0;
  cudaStream_t master = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool dirty = true;
  int* d_step = nullptr;
  std::vector<ForceEntry*> d_ent;
  std::vector<int> n_ent;
  int chunk_cap = 0;
  ForceEntry* h_stage = nullptr;
  size_t h_cap = 0;
  std::vector<char> cls_batched;   // the batching decision the graph was captured with
};

namespace {

void free_ensemble(gt_ensemble* e) {
  if (!e) return;
  cudaSetDevice(e->device);
  if (e->master) cudaStreamSynchronize(e->master);
  if (e->exec) cudaGraphExecDestroy(e->exec);
  if (e->graph) cudaGraphDestroy(e->graph);
  for (auto ev : e->join) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  for (auto p : e->d_ent) if (p) cudaFree(p);
  if (e->d_step) cudaFree(e->d_step);
  if (e->h_stage) cudaFreeHost(e->h_stage);
  for (auto h : e->m) free_handle(h);   // before the slabs their fields live in
  for (auto& c : e->cls) {
    if (c.stream) cudaStreamSynchronize(c.stream);
    if (c.d_ent) cudaFree(c.d_ent);
    if (c.d_count) cudaFree(c.d_count);
    if (c.d_step) cudaFree(c.d_step);
    if (c.btab) cudaFree(c.btab);
    if (c.slab) cudaFree(c.slab);
    if (c.join) cudaEventDestroy(c.join);
    if (c.stream) cudaStreamDestroy(c.stream);
  }
  if (e->master) cudaStreamDestroy(e->master);
  delete e;
}

// Members that can share launches: same grid, box, precision, truncation and
// form of the integrating-factor table.
bool same_class(const gt_params& a, const gt_params& b) {
  return a.nx == b.nx && a.ny == b.ny && a.nz == b.nz && a.precision == b.precision &&
         a.truncate == b.truncate && a.rtrunc == b.rtrunc && a.xlx == b.xlx && a.xly == b.xly &&
         a.xlz == b.xlz;
}

// A class runs batched this chunk when batching is on and all its members
// take the same (pruned or full) path.
bool class_batched(const gt_ensemble* e, const EnsClass& c) {
  if (!e->batching) return false;
  const bool p0 = use_pruning(e->m[c.members[0]]);
  for (int i : c.members)
    if (use_pruning(e->m[i]) != p0) return false;
  return true;
}

template <typename R>
Batch<R> class_batch(const EnsClass& c, const gt_handle* h0) {
  Batch<R> bt;
  bt.nmem = (int)c.members.size();
  bt.mstride = 12 * (long long)h0->g.field_elems();
  bt.emk = reinterpret_cast<const R*>(c.btab);
  bt.emk_len = c.emk_len;
  bt.scal = reinterpret_cast<const R*>(reinterpret_cast<const char*>(c.btab) + c.scal_off);
  return bt;
}

template <typename R>
const DevTables<R>& tables(const gt_handle* h);
template <> const DevTables<float>& tables<float>(const gt_handle* h) { return h->t32; }
template <> const DevTables<double>& tables<double>(const gt_handle* h) { return h->t64; }

// One RK2 step of a whole class: the passes once for all members, then the
// members' forcing of this step.
template <typename R>
int class_step(gt_ensemble* e, EnsClass& c) {
  gt_handle* h0 = e->m[c.members[0]];
  const Batch<R> bt = class_batch<R>(c, h0);
  const int pr = use_pruning(h0) ? 1 : 0;
  CKI(launch_rk2_nlts<R>(h0->g, tables<R>(h0), h0->b, h0->c, h0->w, pr, &h0->pm, h0->d_err, c.stream,
                         hook_fn, h0, &bt));
  if (c.nmax > 0)
    CKI(launch_force_batch<R>(h0->g, h0->b, bt, c.d_ent, c.d_count, c.nmax, kEnsembleChunk, c.d_step,
                              c.stream, hook_fn, h0));
  return GT_OK;
}

int class_enqueue(gt_ensemble* e, EnsClass& c) {
  return e->m[c.members[0]]->mixed ? class_step<float>(e, c) : class_step<double>(e, c);
}

// Builds the classes' batch tables: each member's emk table and its (omega,
// dt, dt2) in the working precision, gathered from the members' own tables.
template <typename R>
int build_batch_tables(gt_ensemble* e, EnsClass& c) {
  const gt_handle* h0 = e->m[c.members[0]];
  const size_t n = c.members.size();
  c.emk_len = h0->ht.emk_by_k2 ? (int)h0->ht.emk_k2.size() : (int)h0->ht.emk_full.size();
  const size_t emk_bytes = n * (size_t)c.emk_len * sizeof(R);
  c.scal_off = (emk_bytes + 255) / 256 * 256;
  CK(cudaMalloc(&c.btab, c.scal_off + 3 * n * sizeof(R)));
  std::vector<R> scal(3 * n);
  for (size_t k = 0; k < n; ++k) {
    const gt_handle* h = e->m[c.members[k]];
    const DevTables<R>& t = tables<R>(h);
    if ((h->ht.emk_by_k2 ? (int)h->ht.emk_k2.size() : (int)h->ht.emk_full.size()) != c.emk_len)
      return GT_EINVAL;
    CK(cudaMemcpy(reinterpret_cast<char*>(c.btab) + k * (size_t)c.emk_len * sizeof(R), t.emk,
                  (size_t)c.emk_len * sizeof(R), cudaMemcpyDeviceToDevice));
    scal[3 * k] = t.omega;
    scal[3 * k + 1] = t.dt;
    scal[3 * k + 2] = t.dt2;
  }
  CK(cudaMemcpy(reinterpret_cast<char*>(c.btab) + c.scal_off, scal.data(), scal.size() * sizeof(R),
                cudaMemcpyHostToDevice));
  return GT_OK;
}

int member_enqueue(gt_ensemble* e, int i) {
  gt_handle* h = e->m[i];
  const int pr = use_pruning(h) ? 1 : 0;
  CKI(rk2_nlts(h, pr));
  if (e->n_ent[i] > 0) {
    if (h->mixed)
      CKI(launch_force_indexed<float>(h->g, h->b, e->d_ent[i], e->n_ent[i], e->d_step + i, h->stream,
                                      hook_fn, h));
    else
      CKI(launch_force_indexed<double>(h->g, h->b, e->d_ent[i], e->n_ent[i], e->d_step + i, h->stream,
                                       hook_fn, h));
  }
  return GT_OK;
}

// The work units of one chunk: batched classes (by class index) and members
// run alone, largest grids first (they are the critical path).
struct Unit {
  int cls;      // >= 0: a batched class
  int member;   // >= 0: a member run alone
  size_t work;
};

std::vector<Unit> work_units(const gt_ensemble* e) {
  std::vector<Unit> u;
  for (size_t k = 0; k < e->cls.size(); ++k) {
    if (!e->cls_batched[k]) continue;
    const gt_handle* h0 = e->m[e->cls[k].members[0]];
    u.push_back({(int)k, -1, h0->g.field_elems() * e->cls[k].members.size()});
  }
  for (size_t i = 0; i < e->m.size(); ++i) {
    const int k = e->cls_of[i];
    if (k >= 0 && e->cls_batched[k]) continue;
    u.push_back({-1, (int)i, e->m[i]->g.field_elems()});
  }
  std::stable_sort(u.begin(), u.end(), [](const Unit& a, const Unit& b) { return a.work > b.work; });
  return u;
}

cudaStream_t unit_stream(gt_ensemble* e, const Unit& u) {
  return u.cls >= 0 ? e->cls[u.cls].stream : e->m[u.member]->stream;
}
cudaEvent_t unit_join(gt_ensemble* e, const Unit& u) {
  return u.cls >= 0 ? e->cls[u.cls].join : e->join[u.member];
}
int unit_enqueue(gt_ensemble* e, const Unit& u) {
  return u.cls >= 0 ? class_enqueue(e, e->cls[u.cls]) : member_enqueue(e, u.member);
}

// Enqueues K steps of every unit: a fork from the master stream, each unit's
// steps on its own stream, a join.
int enqueue_chunk(gt_ensemble* e, int K) {
  CK(cudaEventRecord(e->fork, e->master));
  const std::vector<Unit> units = work_units(e);
  for (const Unit& u : units) CK(cudaStreamWaitEvent(unit_stream(e, u), e->fork, 0));
  for (const Unit& u : units)
    for (int k = 0; k < K; ++k) CKI(unit_enqueue(e, u));
  for (const Unit& u : units) {
    CK(cudaEventRecord(unit_join(e, u), unit_stream(e, u)));
    CK(cudaStreamWaitEvent(e->master, unit_join(e, u), 0));
  }
  return GT_OK;
}

// Captures one chunk (kEnsembleChunk steps of every unit) as a graph.
int build_graph(gt_ensemble* e) {
  if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
  if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
  for (auto h : e->m) h->prof = false;
  CK(cudaStreamBeginCapture(e->master, cudaStreamCaptureModeRelaxed));
  const int rc = enqueue_chunk(e, kEnsembleChunk);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(e->master, &g);
  if (rc) { if (g) cudaGraphDestroy(g); return rc; }
  if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
  e->graph = g;
  CK(cudaGraphInstantiate(&e->exec, e->graph, 0));
  e->dirty = false;
  return GT_OK;
}

}  // namespace

extern "C" {

int gt_ensemble_create(int32_t n, const gt_params* members, gt_ensemble** out) {
  if (n <= 0 || !members || !out) return GT_EINVAL;
  *out = nullptr;
  // every member's parameters and memory budget are checked on the host
  // before anything is allocated
  uint64_t budget = 0;
  gt_get_memory_budget(&budget);
  for (int i = 0; i < n; ++i) {
    if (members[i].device != members[0].device) return GT_EINVAL;
    const int rc = gt_params_validate(&members[i]);
    if (rc) return rc;
    size_t need = 0;
    gt_memory_estimate(&members[i], &need);
    if (budget > 0 && need > budget) {
      set_last_error("ensemble member " + std::to_string(i) + " needs " + std::to_string(need) +
                     " device bytes, over the budget of " + std::to_string(budget));
      return GT_ENOMEM;
    }
  }
  gt_ensemble* e = new (std::nothrow) gt_ensemble();
  if (!e) return GT_ENOMEM;
  e->device = members[0].device;
  cudaError_t ce = cudaSetDevice(e->device);
  if (ce != cudaSuccess) { delete e; return cuda_fail(ce, "cudaSetDevice"); }
  // grid classes of two or more members share a slab of fields
  e->cls_of.assign(n, -1);
  for (int i = 0; i < n; ++i) {
    if (e->cls_of[i] >= 0) continue;
    std::vector<int> mem = {i};
    for (int j = i + 1; j < n; ++j)
      if (e->cls_of[j] < 0 && same_class(members[i], members[j])) mem.push_back(j);
    if (mem.size() < 2) continue;
    EnsClass c;
    c.members = mem;
    for (int j : mem) e->cls_of[j] = (int)e->cls.size();
    e->cls.push_back(c);
  }
  e->m.assign(n, nullptr);
  for (auto& c : e->cls) {
    const gt_params& p0 = members[c.members[0]];
    const size_t esz = p0.precision == GT_PREC_FP64 ? 16 : 8;
    const size_t nh = (size_t)p0.nx / 2 + 1, al = 128 / esz;
    const size_t fbytes = (nh + al - 1) / al * al * p0.ny * p0.nz * esz;
    ce = cudaMalloc(&c.slab, c.members.size() * 12 * fbytes);
    if (ce != cudaSuccess) { free_ensemble(e); return ce == cudaErrorMemoryAllocation ? GT_ENOMEM : cuda_fail(ce, "slab"); }
    for (size_t k = 0; k < c.members.size(); ++k) {
      const int rc = create_handle(&members[c.members[k]], &e->m[c.members[k]],
                                   static_cast<char*>(c.slab) + k * 12 * fbytes);
      if (rc) { free_ensemble(e); return rc; }
      if (e->m[c.members[k]]->g.field_elems() * esz != fbytes) { free_ensemble(e); return GT_EINVAL; }
    }
  }
  for (int i = 0; i < n; ++i) {
    if (e->m[i]) continue;
    const int rc = create_handle(&members[i], &e->m[i], nullptr);
    if (rc) { free_ensemble(e); return rc; }
  }
  ce = cudaStreamCreateWithFlags(&e->master, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  e->join.assign(n, nullptr);
  for (int i = 0; i < n && ce == cudaSuccess; ++i) ce = cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaMalloc(&e->d_step, n * sizeof(int));
  for (auto& c : e->cls) {
    if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaMalloc(&c.d_step, sizeof(int));
  }
  if (ce != cudaSuccess) { free_ensemble(e); return cuda_fail(ce, "gt_ensemble_create"); }
  e->n_ent.assign(n, 0);
  e->d_ent.assign(n, nullptr);
  // entries per step are fixed by each member's forced-mode list
  for (int i = 0; i < n; ++i) {
    gt_handle* h = e->m[i];
    if (h->p.forcing == GT_FORCING_NONE || h->ht.fix.empty()) continue;
    std::vector<ForceEntry> one;
    int32_t seed = 1;
    draw_forcing(h->p, h->ht, seed, one);
    e->n_ent[i] = (int)one.size();
  }
  for (auto& c : e->cls) {
    const int rc = e->m[c.members[0]]->mixed ? build_batch_tables<float>(e, c) : build_batch_tables<double>(e, c);
    if (rc) { free_ensemble(e); return rc; }
    std::vector<int> cnt;
    for (int i : c.members) {
      c.nmax = std::max(c.nmax, e->n_ent[i]);
      cnt.push_back(e->n_ent[i]);
    }
    if (c.nmax > 0) {
      ce = cudaMalloc(&c.d_ent, c.members.size() * kEnsembleChunk * (size_t)c.nmax * sizeof(ForceEntry));
      if (ce == cudaSuccess) ce = cudaMalloc(&c.d_count, cnt.size() * sizeof(int));
      if (ce == cudaSuccess)
        ce = cudaMemcpy(c.d_count, cnt.data(), cnt.size() * sizeof(int), cudaMemcpyHostToDevice);
      if (ce != cudaSuccess) { free_ensemble(e); return cuda_fail(ce, "gt_ensemble_create"); }
    }
  }
  e->cls_batched.assign(e->cls.size(), 0);
  *out = e;
  return GT_OK;
}

int gt_ensemble_destroy(gt_ensemble* e) {
  if (!e) return GT_EINVAL;
  free_ensemble(e);
  return GT_OK;
}

int gt_ensemble_set_state(gt_ensemble* e, int32_t i, const double* bx, const double* by, const double* bz) {
  if (!e || i < 0 || i >= (int)e->m.size()) return GT_EINVAL;
  e->dirty = true;
  return gt_set_state(e->m[i], bx, by, bz);
}

int gt_ensemble_get_state(gt_ensemble* e, int32_t i, double* bx, double* by, double* bz) {
  if (!e || i < 0 || i >= (int)e->m.size()) return GT_EINVAL;
  CK(cudaStreamSynchronize(e->master));
  return gt_get_state(e->m[i], bx, by, bz);
}

int gt_ensemble_energy(gt_ensemble* e, double* energy) {
  if (!e || !energy) return GT_EINVAL;
  CK(cudaStreamSynchronize(e->master));
  for (size_t i = 0; i < e->m.size(); ++i) {
    double ex[3];
    const int rc = gt_energy(e->m[i], ex);
    if (rc) return rc;
    energy[i] = ex[0] + ex[1] + ex[2];
  }
  return GT_OK;
}

int gt_ensemble_autotune(gt_ensemble* e, const char* cache_path) {
  if (!e) return GT_EINVAL;
  CK(cudaStreamSynchronize(e->master));
  // one tuning per distinct (grid, precision) class, applied to every member of the class
  std::vector<std::pair<std::string, Tuning>> done;
  for (auto h : e->m) {
    const std::string key = tuning_key(h);
    bool have = false;
    for (auto& d : done)
      if (d.first == key) { put_tuning(h, d.second); have = true; }
    if (have) continue;
    const int rc = gt_autotune(h, cache_path, nullptr);
    if (rc) return rc;
    done.emplace_back(key, get_tuning(h));
  }
  e->dirty = true;
  return GT_OK;
}

int gt_ensemble_step(gt_ensemble* e, int32_t nsteps, int32_t* seeds, int32_t graph) {
  if (!e || nsteps < 0) return GT_EINVAL;
  const int n = (int)e->m.size();
  bool forced = false;
  for (int i = 0; i < n; ++i) forced = forced || e->n_ent[i] > 0;
  if (forced && !seeds) return GT_EINVAL;
  CK(cudaSetDevice(e->device));
  for (auto h : e->m)
    CK(cudaStreamSynchronize(h->stream));
  // which classes run batched in this call (a change invalidates the graph)
  std::vector<char> bat(e->cls.size());
  for (size_t k = 0; k < e->cls.size(); ++k) bat[k] = class_batched(e, e->cls[k]) ? 1 : 0;
  if (bat != e->cls_batched) {
    e->cls_batched = bat;
    e->dirty = true;
  }
  // pinned staging: members run alone ([K][n_ent] each), then the classes'
  // [member][kEnsembleChunk][nmax] blocks
  size_t total = 0;
  for (int i = 0; i < n; ++i) total += (size_t)kEnsembleChunk * e->n_ent[i];
  for (auto& c : e->cls) total += c.members.size() * (size_t)kEnsembleChunk * c.nmax;
  if (total > e->h_cap) {
    CK(cudaStreamSynchronize(e->master));
    if (e->h_stage) cudaFreeHost(e->h_stage);
    e->h_stage = nullptr;
    e->h_cap = 0;
    CK(cudaMallocHost(&e->h_stage, total * sizeof(ForceEntry)));
    e->h_cap = total;
  }
  if (e->chunk_cap < kEnsembleChunk) {
    for (int i = 0; i < n; ++i) {
      if (e->d_ent[i]) cudaFree(e->d_ent[i]);
      e->d_ent[i] = nullptr;
      if (e->n_ent[i] > 0)
        CK(cudaMalloc(&e->d_ent[i], (size_t)kEnsembleChunk * e->n_ent[i] * sizeof(ForceEntry)));
    }
    e->chunk_cap = kEnsembleChunk;
    e->dirty = true;   // the entry pointers are baked into the graph
  }
  int done = 0;
  while (done < nsteps) {
    const int K = std::min(kEnsembleChunk, nsteps - done);
    CK(cudaStreamSynchronize(e->master));   // the staging buffer and device entries are free
    size_t off = 0;
    std::vector<size_t> cls_off(e->cls.size());
    for (int i = 0; i < n; ++i) off += (size_t)kEnsembleChunk * e->n_ent[i];
    for (size_t k = 0; k < e->cls.size(); ++k) {
      cls_off[k] = off;
      off += e->cls[k].members.size() * (size_t)kEnsembleChunk * e->cls[k].nmax;
    }
    off = 0;
    for (int i = 0; i < n; ++i) {
      const int ne = e->n_ent[i];
      if (ne == 0) continue;
      gt_handle* h = e->m[i];
      std::vector<ForceEntry> steps;
      for (int k = 0; k < K; ++k) {
        const size_t before = steps.size();
        draw_forcing(h->p, h->ht, seeds[i], steps);
        if ((int)(steps.size() - before) != ne || !entries_unique(steps.data() + before, steps.size() - before))
          return GT_EINVAL;
      }
      const int ci = e->cls_of[i];
      if (ci >= 0 && e->cls_batched[ci]) {
        EnsClass& c = e->cls[ci];
        const size_t slot = (size_t)(std::find(c.members.begin(), c.members.end(), i) - c.members.begin());
        for (int k = 0; k < K; ++k)
          std::memcpy(e->h_stage + cls_off[ci] + (slot * kEnsembleChunk + k) * c.nmax,
                      steps.data() + (size_t)k * ne, (size_t)ne * sizeof(ForceEntry));
      } else {
        std::memcpy(e->h_stage + off, steps.data(), steps.size() * sizeof(ForceEntry));
        CK(cudaMemcpyAsync(e->d_ent[i], e->h_stage + off, steps.size() * sizeof(ForceEntry),
                           cudaMemcpyHostToDevice, e->master));
      }
      off += (size_t)kEnsembleChunk * ne;
    }
    for (size_t k = 0; k < e->cls.size(); ++k) {
      EnsClass& c = e->cls[k];
      if (!e->cls_batched[k] || c.nmax == 0) continue;
      CK(cudaMemcpyAsync(c.d_ent, e->h_stage + cls_off[k],
                         c.members.size() * (size_t)kEnsembleChunk * c.nmax * sizeof(ForceEntry),
                         cudaMemcpyHostToDevice, e->master));
      CK(cudaMemsetAsync(c.d_step, 0, sizeof(int), e->master));
    }
    CK(cudaMemsetAsync(e->d_step, 0, n * sizeof(int), e->master));
    if (graph && K == kEnsembleChunk) {
      // one graph launch advances every member by a whole chunk
      if (e->dirty) {
        const int rc = build_graph(e);
        if (rc) return rc;
      }
      CK(cudaGraphLaunch(e->exec, e->master));
    } else {
      const int rc = enqueue_chunk(e, K);
      if (rc) return rc;
    }
    done += K;
  }
  CK(cudaStreamSynchronize(e->master));
  for (auto h : e->m) {
    const int rc = check_device_flag(h);
    if (rc) return rc;
  }
  return GT_OK;
}

int gt_ensemble_set_batching(gt_ensemble* e, int32_t enable) {
  if (!e) return GT_EINVAL;
  e->batching = enable != 0;
  return GT_OK;
}

int gt_ensemble_info(gt_ensemble* e, int32_t* nclasses, int32_t* class_of) {
  if (!e) return GT_EINVAL;
  if (nclasses) *nclasses = (int32_t)e->cls.size();
  if (class_of)
    for (size_t i = 0; i < e->m.size(); ++i) class_of[i] = e->cls_of[i];
  return GT_OK;
}

}  // extern "C"
