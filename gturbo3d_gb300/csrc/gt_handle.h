// Private to the C-ABI translation units (core, autotuner, tangent-linear and
// adjoint, ensemble): the handle behind the opaque gt_handle of the public
// header and the helpers those units share.
#pragma once

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gt_internal.h"

namespace gtc {

// Records "what: CUDA error string" as the thread's last error; GT_ECUDA.
int cuda_fail(cudaError_t e, const char* what);

// One profiled launch: its kind and the events around it.
struct Pending {
  int kind;
  cudaEvent_t e0, e1;
};

}  // namespace gtc

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return gtc::cuda_fail(e_, #call); \
  } while (0)

#define CKI(rcexpr)                                                  \
  do {                                                               \
    int r_ = (rcexpr);                                               \
    if (r_ != 0) return gtc::cuda_fail((cudaError_t)r_, #rcexpr);         \
  } while (0)

struct gt_handle {
  gt_params p{};
  gt::HostTables ht;
  gt::Geom g{};
  int mixed = 0;
  int csize = 16;
  cudaStream_t stream = nullptr;
  void* fields_mem = nullptr;
  bool owns_fields = true;     // false: the fields live in an ensemble class slab
  void* b[3]{};
  void* c[3]{};
  void* w[6]{};
  void* stage = nullptr;       // one FP64 spectral field [nz][ny][nhp] double2
  void* tab_mem = nullptr;
  gt::DevTables<double> t64{};
  gt::DevTables<float> t32{};
  // forcing entries: double-buffered pinned staging and device buffers
  gt::ForceEntry* d_force[2]{};
  gt::ForceEntry* h_force[2]{};
  size_t force_cap[2]{};
  cudaEvent_t force_copied[2]{};
  int force_slot = 0;
  double* d_partials = nullptr;
  int npartials = 0;
  double* d_result = nullptr;
  double* h_result = nullptr;
  int* h_flag = nullptr;       // pinned: the device error flag read back with the results
  int nresult = 0;
  int64_t launches = 0;
  // truncation-aware pruning: allowed by the caller, the state is zero outside
  // the kept set K, and every forced mode lies in K
  bool prune_enabled = true;
  bool state_in_k = false;
  bool forcing_in_k = false;
  unsigned long long* d_count = nullptr;
  // launch-shape knobs, and the device error flag that bounded device waits raise
  gt::PassTuning pm{};
  int* d_err = nullptr;
  bool prof = false;
  std::vector<gtc::Pending> pending;
  std::vector<cudaEvent_t> pool;
  int64_t kind_launches[gt::kNumKinds]{};
  double kind_ms[gt::kNumKinds]{};
};

namespace gtc {

// Launch hook of every kernel: counts launches and, when profiling, brackets
// them with events.
void hook_fn(void* ctx, int kind, bool begin);
// One nonlinear term in the handle's precision.
int nlt(gt_handle* h, void* const a[3], void* const bcor[3], void* const out[3], int mode,
        int pruned = 0);
// Both nonlinear terms of one RK2 step, b -> c -> b.
int rk2_nlts(gt_handle* h, int pruned);
// Reads and clears the device error flag of the bounded waits.
int check_device_flag(gt_handle* h);
// The same for a flag already copied into h->h_flag and synchronised.
int take_device_flag(gt_handle* h);
// The truncation-aware pruned passes apply (allowed, truncating, state and
// forcing inside the kept set).
bool use_pruning(const gt_handle* h);
// Host FP64 half spectrum [nz][ny][nh] <-> a device field in working precision.
int upload_spec(gt_handle* h, const double* host, void* dst);
int download_spec(gt_handle* h, const void* src, double* host);
// Enqueues nsteps RK2 steps; all[offs[s] .. offs[s+1]) are step s's forcing adds.
int run_steps(gt_handle* h, int nsteps, const std::vector<gt::ForceEntry>& all,
              const std::vector<size_t>& offs);
// Makes the handle's device current and clears a stale non-sticky error.
int set_dev(gt_handle* h);
void free_handle(gt_handle* h);
// gt_create, with the twelve fields optionally in caller-owned device memory.
int create_handle(const gt_params* p, gt_handle** out, void* ext_fields);

// Launch-shape knobs the autotuner searches.
struct Tuning {
  int y_tx, z_tx, x_fused, y_pairs, fuse_stage, z_split, y_prefetch, overlap, slab_pipe, zf_pipe;
};

Tuning get_tuning(const gt_handle* h);
void put_tuning(gt_handle* h, const Tuning& t);
// Cache key: grid, precision, pruning and GPU name.
std::string tuning_key(const gt_handle* h);
// Coordinate descent over the knobs; the choice is cached in cache_path.
int autotune_handle(gt_handle* h, const char* cache_path, double* best_ms_out);

}  // namespace gtc
