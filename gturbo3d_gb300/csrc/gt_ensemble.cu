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
// advanced together; in graph mode one CUDA graph launch advances every member
// by one step (each member's kernels on its own stream, forked and joined in
// the graph), with the forcing drawn on the host per chunk of steps and read
// on the device by step index.
// ===========================================================================
struct gt_ensemble {
  std::vector<gt_handle*> m;
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
};

namespace {

constexpr int kEnsembleChunk = 64;

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
  for (auto h : e->m) free_handle(h);
  if (e->master) cudaStreamDestroy(e->master);
  delete e;
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

// Members by decreasing grid size: the largest members are the critical
// path, so their work is issued first.
std::vector<int> launch_order(const gt_ensemble* e) {
  std::vector<int> order(e->m.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return e->m[a]->g.field_elems() > e->m[b]->g.field_elems();
  });
  return order;
}

// Captures one chunk (kEnsembleChunk steps) of every member: a fork, each
// member's steps on its own stream, a join.  Members progress independently
// within the chunk; the only barrier is the join at its end.
int build_graph(gt_ensemble* e) {
  if (e->exec) { cudaGraphExecDestroy(e->exec); e->exec = nullptr; }
  if (e->graph) { cudaGraphDestroy(e->graph); e->graph = nullptr; }
  for (auto h : e->m) h->prof = false;
  CK(cudaStreamBeginCapture(e->master, cudaStreamCaptureModeRelaxed));
  int rc = GT_OK;
  cudaEventRecord(e->fork, e->master);
  for (int i : launch_order(e)) {
    if (rc) break;
    cudaStreamWaitEvent(e->m[i]->stream, e->fork, 0);
    for (int k = 0; k < kEnsembleChunk && !rc; ++k) rc = member_enqueue(e, i);
    cudaEventRecord(e->join[i], e->m[i]->stream);
    cudaStreamWaitEvent(e->master, e->join[i], 0);
  }
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
  for (int i = 0; i < n; ++i) {
    if (members[i].device != e->device) { free_ensemble(e); return GT_EINVAL; }
    gt_handle* h = nullptr;
    const int rc = gt_create(&members[i], &h);
    if (rc) { free_ensemble(e); return rc; }
    e->m.push_back(h);
  }
  cudaSetDevice(e->device);
  cudaError_t ce = cudaStreamCreateWithFlags(&e->master, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  e->join.assign(n, nullptr);
  for (int i = 0; i < n && ce == cudaSuccess; ++i) ce = cudaEventCreateWithFlags(&e->join[i], cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaMalloc(&e->d_step, n * sizeof(int));
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
  int done = 0;
  while (done < nsteps) {
    const int K = std::min(kEnsembleChunk, nsteps - done);
    // draw and upload K steps of forcing per member
    size_t total = 0;
    for (int i = 0; i < n; ++i) total += (size_t)K * e->n_ent[i];
    CK(cudaStreamSynchronize(e->master));   // the staging buffer is free
    if (total > e->h_cap) {
      if (e->h_stage) cudaFreeHost(e->h_stage);
      e->h_stage = nullptr;
      e->h_cap = 0;
      CK(cudaMallocHost(&e->h_stage, total * sizeof(ForceEntry)));
      e->h_cap = total;
    }
    if (K > e->chunk_cap) {
      for (int i = 0; i < n; ++i) {
        if (e->d_ent[i]) cudaFree(e->d_ent[i]);
        e->d_ent[i] = nullptr;
        if (e->n_ent[i] > 0)
          CK(cudaMalloc(&e->d_ent[i], (size_t)kEnsembleChunk * e->n_ent[i] * sizeof(ForceEntry)));
      }
      e->chunk_cap = kEnsembleChunk;
      e->dirty = true;   // the entry pointers are baked into the graph
    }
    size_t off = 0;
    for (int i = 0; i < n; ++i) {
      if (e->n_ent[i] == 0) continue;
      gt_handle* h = e->m[i];
      std::vector<ForceEntry> steps;
      for (int k = 0; k < K; ++k) {
        const size_t before = steps.size();
        draw_forcing(h->p, h->ht, seeds[i], steps);
        if ((int)(steps.size() - before) != e->n_ent[i] ||
            !entries_unique(steps.data() + before, steps.size() - before))
          return GT_EINVAL;
      }
      std::memcpy(e->h_stage + off, steps.data(), steps.size() * sizeof(ForceEntry));
      CK(cudaMemcpyAsync(e->d_ent[i], e->h_stage + off, steps.size() * sizeof(ForceEntry),
                         cudaMemcpyHostToDevice, e->master));
      off += steps.size();
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
      // one launch sequence per member and step, each member on its own stream
      CK(cudaEventRecord(e->fork, e->master));
      for (int i = 0; i < n; ++i) CK(cudaStreamWaitEvent(e->m[i]->stream, e->fork, 0));
      const std::vector<int> order = launch_order(e);
      for (int k = 0; k < K; ++k)
        for (int i : order) {
          const int rc = member_enqueue(e, i);
          if (rc) return rc;
        }
      for (int i = 0; i < n; ++i) {
        CK(cudaEventRecord(e->join[i], e->m[i]->stream));
        CK(cudaStreamWaitEvent(e->master, e->join[i], 0));
      }
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

}  // extern "C"
