// Internal declarations shared by the host set-up code (gt_host.cpp), the
// kernels (gt_kernels_impl.cuh, compiled once per precision) and the C-ABI
// (gt_capi.cu, gt_autotune.cu, gt_tl_adj.cu, gt_ensemble.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>


#include "../../include/gturbo_gb.h"

namespace gt {

constexpr double kPiRef = 3.14159265358979323846;          // defk.f90:24
constexpr double kPi2_3d3c = 2.0 * 3.14159265358979323846; // forcing_3d3c.f90:21
constexpr double kPi2_2d2c = 2.0 * 3.14159265358979;       // forcing_2d2c.f90:20
constexpr int32_t kLcgMul = 69069;                          // forcing_3d3c.f90:89
constexpr int32_t kLcgMask = 0x7FFFFFFF;                    // forcing_3d3c.f90:88

// Wavenumber tables and derived per-mode data, as defk builds them
// (defk.f90:13-91), plus the truncation boundary and forced-mode list.
struct HostTables {
  int nx = 0, ny = 0, nz = 0, nh = 0;
  std::vector<double> fkx, fky, fkz, fkxs, fkys, fkzs;
  std::vector<int32_t> jc, kc;                 // 0-based conjugate indices
  double fkxsmax = 0, fkysmax = 0, fkzsmax = 0, rtrunc2 = 0;
  // emk = exp(-0.5 dt (nu k2^alpnu + mu k2^alpmu)), = 1 at k2 = 0.
  bool emk_by_k2 = false;                      // integer wavenumbers: emk indexed by k2
  std::vector<double> emk_k2;                  // [k2max + 1] when emk_by_k2
  std::vector<double> emk_full;                // [nz][ny][nh] otherwise
  // Truncation: mode (ix, iy, iz) survives trunc iff ix < xcut[iz*ny + iy]
  // (and it is not (0,0,0)).  xcut = nh everywhere when truncate = 0.
  std::vector<int32_t> xcut;
  // Forced modes in the reference's order.
  std::vector<int32_t> fix, fiy, fiz;
  std::vector<double> ff;
  double inpe = 0, inpz = 0;
};

// One scatter-add of the forcing: b_c(z, y, x) += inc[2c] + i inc[2c+1] for
// every component c whose bit is set in mask.
struct ForceEntry {
  int32_t z, y, x, mask;
  double inc[6];
};

int build_tables(const gt_params& p, HostTables& t);
// Records the text gt_last_error() returns on the calling thread.
void set_last_error(const std::string& msg);
double emk_value(const gt_params& p, double k2);
// rann (forcing_3d3c.f90:82-93): advance state, return REAL*4 value.
float rann(int32_t& irand);
// Appends one step's forcing entries, in the reference's order, advancing
// the seed exactly as forcing_3d3c.f90:26-72 / forcing_2d2c.f90:27-48 do.
void draw_forcing(const gt_params& p, const HostTables& t, int32_t& seed,
                  std::vector<ForceEntry>& out);
bool entries_unique(const ForceEntry* e, size_t n);

// ---- device side --------------------------------------------------------

// Layout of one spectral field on the device: [nz][ny][nhp] complex with the
// row length nhp padded to a multiple of 128 bytes.
struct Geom {
  int nx, ny, nz, nh, nhp;
  int lnx, lny, lnz;  // log2 of nx, ny, nz
  size_t field_elems() const { return (size_t)nz * ny * nhp; }
};

// Device-resident tables, in the working precision R (float or double)
// except where noted.
template <typename R>
struct DevTables {
  const R* fkx;    // [nh]
  const R* fky;    // [ny]
  const R* fkz;    // [nz]
  const R* fkxs;   // [nh]
  const R* fkys;   // [ny]
  const R* fkzs;   // [nz]
  const R* emk;    // by k2 (emk_by_k2) or [nz][ny][nh]
  int emk_by_k2;
  const int32_t* xcut;  // [nz][ny]
  const void* twx;      // twiddles exp(-2 pi i m / nx), m < nx  (complex R)
  const void* twy;      // ny
  const void* twz;      // nz
  const void* twzh;     // nz / 2 (the half-length z transforms of the cluster-pair z passes)
  R omega, dt, dt2, scale;  // scale = 1/(nx ny nz)
  int truncate;
  // Truncation-aware pruning (truncate = 1 and a state that is zero outside
  // the kept set K): column (X, y) holds nonzero modes only if X < xcut[y]
  // (the z = 0 row of xcut); ztiles lists the (x-tile, y) blocks of the z
  // passes that contain such a column; xa = xcut[0] bounds every kept kx.
  const int32_t* ztiles;   // pairs (x-tile, y) for the default z tile width
  int nztiles;
  const int32_t* ztl[11];  // the same for every tile width 2^lg, lg = 0..10
  int nztl[11];
  const int32_t* ztlzc[11];  // per entry of ztl[lg]: the largest z <= nz/2 whose row keeps the
                             // tile's first column (the kept z are z <= zc and z >= nz - zc)
  int xa;
};

enum NltMode { kNltOnly = 0, kStage1 = 1, kStage2 = 2 };

// Members of one ensemble grid class advanced by the same launches: the
// members' fields lie in one slab, member m's field f at member 0's field f
// plus m * mstride elements; each member has its own integrating factor
// (emk tables emk_len apart) and scalars (omega, dt, dt2 at scal[3 m]).  The
// member index is a spare grid axis of every pass kernel.  nmem = 0: one
// member, the launch of a single handle.
template <typename R>
struct Batch {
  int nmem = 0;
  long long mstride = 0;
  const R* emk = nullptr;
  int emk_len = 0;
  const R* scal = nullptr;
};

// Launch-shape knobs of the passes (the gt_set_tuning keys); every setting
// gives the same result up to rounding.
struct PassTuning {
  int y_tx = 0, z_tx = 0;   // tile width of the y / z passes (0: default)
  int y_pairs = 1;          // FP32 y passes: 1 = two adjacent columns per thread
  int y_prefetch = 1;       // FP32 y passes (with y_pairs) as persistent blocks that double-buffer
                            // their tiles with asynchronous copies: 0 = neither, 1 = the inverse
                            // pass (default: 0.90 -> 0.84 ms at 512^3), 2 = both (the forward
                            // pass measured slower: 0.37 -> 0.42 ms)
  int x_fused = 2;          // x pass: 2 = one thread group per row pair, a row's three lines
                            // transformed together; 3 = the same with row 0's products
                            // parked in shared memory (the default for FP32 at NX = 512);
                            // 1 = the lines one by one; 0 = three groups per row pair
  int fuse_stage = 0;       // RK2 step: 1 = fused z forward + z inverse at the stage boundary
  int z_split = 0;          // z inverse pass: 1 = curl part and k^2 part in separate kernels;
                            // 2 = one one-region kernel, inputs read again per output line
  int overlap = 0;          // 1 = the k^2 half of the z inverse pass and the inverse y transforms
                            // of its three fields on a second stream, concurrently with the curl
                            // half and the y transforms of u (needs stream2 and the two events)
  int zf_pipe = 0;          // 1 = the z forward pass persistent, the next tile's inputs copied
                            // asynchronously behind the current tile's epilogue
  int slab_pipe = 0;        // 1 = the y inverse, x and y passes over two halves of the z-planes on
                            // two streams, the second half's y inverse after the first half's
  int z_tma = 0;            // FP32, z columns of up to 512 points, tiles loaded by TMA (one thread
                            // issues them, an mbarrier per field): bit 1 = the z forward pass, bit 2
                            // = the z inverse pass (both the default for z columns of 256 and 512);
                            // bit 4, with bit 2: the z inverse pass's outputs leave by TMA stores
                            // (the default for z columns of 256)
  int z_cluster = 0;        // FP32: 1 = the z forward pass on cluster pairs of CTAs, each holding half
                            // of a tile's z-rows (two tiles per SM; the default for z columns of 1024
                            // points or more); 0 = one CTA per tile
  void* stream2 = nullptr;  // the handle's second stream and the events for overlap / slab_pipe
  void* ev_fork = nullptr;
  void* ev_join = nullptr;
  void* ev_mid = nullptr;
};

// Work buffers: w[0..5] hold u_x,u_y,u_z,w_x,w_y,w_z between passes; after
// the x-pass w[0..2] hold u x w.
template <typename R>
struct Fields {
  void* b[3];
  void* c[3];
  void* w[6];
};

// Launchers (gt_kernels_impl.cuh).  All enqueue on `s` and return cudaError_t as int.
struct LaunchRec;  // profiling hook
using LaunchHook = void (*)(void* ctx, int kind, bool begin);

enum KernelKind {
  kKZinvCurl = 0, kKYPass, kKXCross, kKZFwdEpi, kKForce, kKConvert, kKDiag, kKDiagFinal,
  kKFft1, kKPoint, kKYFwd, kKZFwdZinv, kNumKinds
};
const char* kernel_kind_name(int k);

template <typename R>
int launch_rk2_nlts(const Geom& g, const DevTables<R>& tb, void* const b[3], void* const c[3],
                    void* const w[6], int pruned, const PassTuning* pm, int* err, void* stream,
                    LaunchHook hook, void* hctx, const Batch<R>* bt = nullptr);
template <typename R>
int launch_nlt(const Geom& g, const DevTables<R>& tb, void* const a[3], void* const bcor[3],
               void* const out[3], void* const w[6], int mode, int pruned, const PassTuning* pm,
               int* err, void* stream, LaunchHook hook, void* hctx);
int launch_wait_selftest(int* err, void* stream);
// (x-tile, y) blocks of the pruned z passes for precision with complex size csize.
void build_ztiles(const Geom& g, const int32_t* xcut, int csize, std::vector<int32_t>& tiles,
                  int tx = 0);
// Number of state values (over 3 fields) that are nonzero at modes outside K.
template <typename R>
int launch_count_outside(const Geom& g, const DevTables<R>& tb, void* const b[3],
                         unsigned long long* d_count, void* stream);
template <typename R>
int launch_force(const Geom& g, void* const b[3], const ForceEntry* entries, int n, int serial,
                 void* stream, LaunchHook hook, void* hctx);
// Forcing of a grid class's members at step *step: member m adds its first
// count[m] entries of base[(m * nsteps + *step) * nmax ...], then ++*step.
template <typename R>
int launch_force_batch(const Geom& g, void* const b[3], const Batch<R>& bt, const ForceEntry* base,
                       const int* count, int nmax, int nsteps, const int* step, void* stream,
                       LaunchHook hook, void* hctx);
// Forcing of step *step from resident per-step entries, then ++*step.
template <typename R>
int launch_force_indexed(const Geom& g, void* const b[3], const ForceEntry* base, int n,
                         const int* step, void* stream, LaunchHook hook, void* hctx);
// Field conversions between the device FP64 staging layout [nz][ny][nhp]
// double2 and the working precision.
template <typename R>
int launch_convert(const Geom& g, const void* src, void* dst, int to_working, void* stream,
                   LaunchHook hook, void* hctx);
// Plain 3D transforms of one field (real layout [nz][ny][nx] in w-buffers).
template <typename R>
int launch_fft_inv(const Geom& g, const DevTables<R>& tb, void* spec, void* real_out,
                   void* const w[6], void* stream, LaunchHook hook, void* hctx);
template <typename R>
int launch_fft_dir(const Geom& g, const DevTables<R>& tb, const void* real_in, void* spec_out,
                   void* const w[6], void* stream, LaunchHook hook, void* hctx);
// Pointwise spectral ops used by the output and initial-state paths.
// op: 0 = curl, 1 = invcurl, 2 = trunc, 3 = incompr (writes |k.a|^2 partials)
template <typename R>
int launch_point(const Geom& g, const DevTables<R>& tb, void* const a[3], int op, double* partial,
                 int npartial, void* stream, LaunchHook hook, void* hctx);

// Diagnostics: per-CTA partials then a fixed-order final reduction.
constexpr int kDiagScalars = 20;  // 9 energy, 9 enstrophy, helicity, nonfinite
template <typename R>
int launch_diag(const Geom& g, const DevTables<R>& tb, void* const b[3], void* const n1[3],
                double nu, double alpnu, double mu, double alpmu, double* partials, int nblocks,
                double* result /* kDiagScalars + 3*nbin */, void* stream, LaunchHook hook,
                void* hctx);
template <typename R>
int launch_energy(const Geom& g, const DevTables<R>& tb, void* const b[3], int pruned, double* partials,
                  int nblocks, double* result, void* stream, LaunchHook hook, void* hctx);
int diag_blocks(const Geom& g);
// Tangent-linear / adjoint building blocks (gt_adjoint.cu): out = op(a) [+ beta b].
template <typename R>
int launch_spec_op(const Geom& g, const DevTables<R>& tb, void* const out[3], void* const a[3],
                   void* const b[3], int op, double sgn, double kmin2, double beta, void* stream);
template <typename R>
int launch_phys_cross(const Geom& g, void* const out[3], void* const a[3], void* const b[3],
                      void* const c[3], void* const d[3], double s1, double s2, void* stream);

}  // namespace gt
