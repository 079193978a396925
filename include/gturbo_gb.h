/*
 * gturbo_gb.h -- C-ABI of the GB300-native RK2 integrating-factor step of
 * Gturbo3D (triply periodic rotating Navier-Stokes, vector-potential form).
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (GT_OK = 0, a negative GT_E* code otherwise) and never throws.
 * A handle owns its device memory and one CUDA stream; calls on one handle
 * must not overlap (a handle is not thread-safe).  Host arrays passed in are
 * borrowed only for the duration of the call.
 *
 * Spectral arrays on the host use the reference layout: complex*16
 * (NX/2+1, NY, NZ) with x fastest, i.e. double[NZ][NY][NX/2+1][2] in C order
 * (main.f90:14).  Physical arrays are double[NZ][NY][NX] (the reference's
 * real*8 (NX+2, NY, NZ) without its two padding columns).
 *
 * There is no CPU fallback: compute entry points fail with GT_ECUDA when no
 * GPU is usable.  The host-only entry points (marked "host only") run
 * without a GPU.
 */
#ifndef GTURBO_GB_H
#define GTURBO_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GT_OK 0
#define GT_EINVAL (-1)       /* bad argument or parameter                      */
#define GT_ENOMEM (-2)       /* device or host allocation failed / over budget */
#define GT_ECUDA (-3)        /* CUDA runtime error (no device, launch failure) */
#define GT_ENFORC (-4)       /* more forced modes than NFORC (iniforcing_3d3c.f90:33) */
#define GT_ENONFINITE (-5)   /* state holds NaN or Inf                         */
#define GT_EIO (-6)          /* file missing, unreadable or malformed          */
#define GT_ETIMEOUT (-7)     /* a bounded device wait ran out                  */

/* ---- enumerations ---------------------------------------------------- */
#define GT_FORCING_NONE 0
#define GT_FORCING_3D3C 1    /* forcing_3d3c.f90 / iniforcing_3d3c.f90 */
#define GT_FORCING_2D2C 2    /* forcing_2d2c.f90 / iniforcing_2d2c.f90 */

#define GT_DT2_AS_BUILT 0    /* dt2 = 0: rkstep.f90 reads a dt2 nothing assigns */
#define GT_DT2_RK2 1         /* dt2 = dt/2: the RK2 midpoint the scheme intends  */

#define GT_PREC_FP64 0       /* plain form: everything in FP64                    */
#define GT_PREC_MIXED 1      /* FP32 state, FFTs and products; FP64 exponentials,
                                forcing normalisation and reductions             */

#define GT_NFORC 2048        /* modules.f90:38 */

/* ---- parameters ------------------------------------------------------- */
/* The values main.f90 reads from params.dat (inieuler.f90:14-20), the
 * compile-time grid (modules.f90:4, here a runtime value), the link-time
 * forcing variant (Makefile:20-33) and the choices the reference leaves
 * implicit. */
typedef struct gt_params {
  int32_t nx, ny, nz;          /* powers of two, 8..1024 each                 */
  double xlx, xly, xlz;        /* box lengths                                 */
  double nu, alpnu, mu, alpmu; /* hyper-viscosity and friction                */
  double dt, omega;            /* time step; Coriolis coefficient (nlt.f90:67-81) */
  double rtrunc;               /* truncation radius, NOT squared (defk.f90:91 squares it) */
  int32_t truncate;            /* 1: 2/3-rule dealiasing on                   */
  double famp, k1f, k2f;       /* forcing amplitude and shell k1f < |k| <= k2f */
  int32_t forcing;             /* GT_FORCING_*                                */
  int32_t dt2_mode;            /* GT_DT2_*                                    */
  int32_t precision;           /* GT_PREC_*                                   */
  int32_t device;              /* CUDA device ordinal                         */
} gt_params;

/* Global diagnostics (diagnostics.f90:114-199 plus helicity).  energy[] and
 * enstrophy[] hold, in order: the x, y, z components; the viscous
 * dissipation 2 nu sum fac |.|^2 k^(2 alpnu) per component; the friction
 * dissipation per component.  fac = 1/2 on the kx = 0 and kx = NX/2 planes. */
typedef struct gt_diag {
  double energy[9];
  double enstrophy[9];
  double helicity;             /* sum fac Re(u . conj(w)), k != 0 (no reference counterpart) */
  double inpe, inpz;           /* mean energy / enstrophy input of the forcing */
  int64_t nonfinite;           /* number of non-finite state values            */
} gt_diag;

typedef struct gt_handle gt_handle;

/* ---- host only ---------------------------------------------------------- */
/* Fills the reference's params.dat defaults for a 2 pi box (params.dat:1-6). */
int gt_params_default(gt_params* p);
/* Checks a parameter set (grid sizes, positivity, enum values). */
int gt_params_validate(const gt_params* p);
/* Reads params.dat's six list-directed lines (inieuler.f90:14-20) into p;
 * fields not in the file keep their values.  GT_EIO on a missing or
 * malformed file. */
int gt_params_read(const char* path, gt_params* p);
/* Device bytes gt_create would allocate for p. */
int gt_memory_estimate(const gt_params* p, size_t* bytes);
/* Process-wide cap on the device bytes one handle may allocate (0 = no cap,
 * the default).  gt_create (and every member of gt_ensemble_create) whose
 * gt_memory_estimate exceeds it returns GT_ENOMEM before any CUDA call, so
 * a driver that shares the GPU with other work can bound the library's
 * footprint.  The reference has no counterpart: its arrays are static and
 * an oversized grid fails at load or allocation time.  Host only. */
int gt_set_memory_budget(uint64_t bytes);
int gt_get_memory_budget(uint64_t* bytes);
/* One draw of the reference's rann (forcing_3d3c.f90:82-93): advances
 * *irand and writes REAL*4(irand / (2^31-1)).  n draws in a row. */
int gt_rann(int32_t* irand, int32_t n, float* out);
/* Forced-mode list in the reference's order (iniforcing_3d3c.f90:22-184 or
 * iniforcing_2d2c.f90:14-67).  0-based indices; arrays must hold GT_NFORC
 * entries (any may be NULL).  GT_ENFORC if the list would exceed GT_NFORC. */
int gt_forced_modes(const gt_params* p, int32_t* nf, int32_t* ix, int32_t* iy, int32_t* iz,
                    double* ff, double* inpe, double* inpz);
/* One step's forcing increments exactly as forcing_3d3c.f90:26-72 or
 * forcing_2d2c.f90:27-43 compute them, drawn with rann from *seed (which is
 * advanced).  Writes n entries (mode iz[e], iy[e], ix[e]; dF[e*6 + 2c],
 * dF[e*6 + 2c + 1] = Re, Im of the increment of component c), in the order
 * the reference adds them, including the conjugate partners on the kx = 0
 * and kx = NX/2 planes; cap bounds the arrays (2*GT_NFORC always suffices).
 * Feed them to gt_rk2_step_coeffs for host-driven forcing. */
int gt_forcing_increments(const gt_params* p, int32_t* seed, int32_t cap, int32_t* n,
                          int32_t* ix, int32_t* iy, int32_t* iz, double* dF);
/* The reference's initial noise for a fresh start (inieuler.f90:76-82,
 * trunc.f90:75-93): u_c = sqrt(dt) * (rann(seed) - 0.5) at every point, the
 * three components of a point drawn in turn, points in Fortran order (x
 * fastest), REAL*4 difference promoted to REAL*8.  Writes double[NZ][NY][NX]
 * each and advances *seed by 3 NX NY NZ draws; feed the result to
 * gt_set_state_physical (main.f90:91-106).  Host only. */
int gt_init_noise(const gt_params* p, int32_t* seed, double* ux, double* uy, double* uz);
/* Reads / writes the seed file files/seed.NNN (main.f90:40-45, 207-210). */
int gt_seed_read(const char* path, int32_t* seed);
int gt_seed_write(const char* path, int32_t seed);
/* Reads / writes curframe.dat, the frame number and time a continuation
 * starts from (main.f90:37-39, 212-215).  Host only. */
int gt_frame_read(const char* path, int32_t* ifr, double* t);
int gt_frame_write(const char* path, int32_t ifr, double t);
/* Reads / writes one float32 real-space field as a Fortran unformatted
 * sequential record of NX*NY*NZ values, x fastest (read.f90:12-52,
 * write.f90:12-22). */
int gt_field_read_f32(const char* path, int32_t nx, int32_t ny, int32_t nz, float* out);
int gt_field_write_f32(const char* path, int32_t nx, int32_t ny, int32_t nz, const float* in);

/* ---- handle ------------------------------------------------------------- */
/* Builds the wavenumber tables and integrating factor (defk.f90:13-91), the
 * forced-mode list (iniforcing_*.f90), the FFT twiddle tables, and
 * allocates the device state.  The initial state is zero. */
int gt_create(const gt_params* p, gt_handle** out);
int gt_destroy(gt_handle* h);
/* Spectral vector potential b in the host layout described above. */
int gt_set_state(gt_handle* h, const double* bx, const double* by, const double* bz);
int gt_get_state(gt_handle* h, double* bx, double* by, double* bz);

/* Drop-in for the body of main.f90:121-150, nsteps times: N1 = nlt(b);
 * c = step1(b, N1); N2 = nlt(c; Coriolis from b); b = step2(b, N2);
 * forcing(b, seed).  The forcing draws are made on the host with the
 * reference's rann, advancing *seed_inout exactly as the reference's
 * device-resident seed advances.  seed_inout may be NULL when forcing is
 * GT_FORCING_NONE. */
int gt_rk2_step(gt_handle* h, int32_t nsteps, int32_t* seed_inout);
/* One RK2 step with caller-supplied forcing: after step2, adds for each of
 * n entries the complex increments dF[e*6 + 2c], dF[e*6 + 2c + 1] (component
 * c = x, y, z) at mode (iz[e], iy[e], ix[e]), in entry order. */
int gt_rk2_step_coeffs(gt_handle* h, int32_t n, const int32_t* ix, const int32_t* iy,
                       const int32_t* iz, const double* dF);
/* Nonlinear term N = nlt(a; Coriolis source = current state) (nlt.f90:1-95)
 * for a host-supplied a; writes N to the host arrays. */
int gt_nonlinear(gt_handle* h, const double* ax, const double* ay, const double* az,
                 double* nx_out, double* ny_out, double* nz_out);
/* Diagnostics of the current state: glob (diagnostics.f90:114-199),
 * helicity, spectrum E(k) and E2D(k) (diagnostics.f90:5-56) and the flux
 * Pi(k) (diagnostics.f90:62-103, evaluated with N1 = nlt(b)).  ek, ek2d and
 * flux hold NX/2 values each and may be NULL (flux = NULL skips the extra
 * nlt).  Reductions are FP64 and in a fixed order (bitwise reproducible). */
int gt_diagnostics(gt_handle* h, gt_diag* out, double* ek, double* ek2d, double* flux);
/* Kinetic energy of the current state per component, E_c = sum_{k != 0}
 * fac |(i k x b)_c|^2 (the energy terms of diagnostics.f90:126-138) in FP64,
 * by a fixed-order reduction: the cheap per-step observable. */
int gt_energy(gt_handle* h, double* energy_xyz);
/* 3D transforms of one field through the library's FFT passes:
 * gt_fft_dir = fft_dir.f90 (R2C scaled by 1/(NX NY NZ)),
 * gt_fft_inv = fft_inv.f90 (unnormalised C2R). */
int gt_fft_dir(gt_handle* h, const double* real_in, double* spec_out);
int gt_fft_inv(gt_handle* h, const double* spec_in, double* real_out);
/* Velocity u = curl b in physical space (the output path main.f90:188-201). */
int gt_velocity(gt_handle* h, double* ux, double* uy, double* uz);
/* Initial-state path (main.f90:91-106): from a physical velocity field, b =
 * trunc(invcurl(incompr(fft_dir(u)))).  *cc (may be NULL) receives the
 * removed compressibility sum |k.u|^2 (trunc.f90:47-64). */
int gt_set_state_physical(gt_handle* h, const double* ux, const double* uy, const double* uz,
                          double* cc);
/* GT_ENONFINITE if the state holds a NaN or Inf, GT_OK otherwise. */
int gt_check_finite(gt_handle* h);
/* Truncation-aware pruning of the time step (on by default).  With
 * truncate = 1 the state and every nonlinear term live on the kept set K of
 * trunc.f90:14-17; the step then skips the FFT lines and modes that are zero
 * and returns the same result up to rounding.  It is used only while the
 * state is zero outside K (checked on every gt_set_state*, and kept by the
 * step itself) and every forced mode lies in K. */
int gt_set_pruning(gt_handle* h, int32_t enable);
/* *active = 1 if the next gt_rk2_step takes the pruned path. */
int gt_pruning_active(gt_handle* h, int32_t* active);
/* Launch-shape tuning (results are unchanged):
 * "y_tx", "z_tx" (0 = default, or 2/4/8/16: x-columns per block of the y / z passes;
 * the z default is 16 for FP32 z columns of 256 points or more, else 8),
 * "x_fused" (x pass: 2 = one thread group per row pair, the three packed lines
 * of a row transformed together, u x w in registers (default); 3 = the same
 * with row 0's products parked in shared memory, three resident blocks per SM
 * (the default for the mixed form at NX = 512);
 * 1 = the lines transformed one by one; 0 = three groups per row pair),
 * "y_pairs" (0/1: FP32 y passes with
 * two adjacent columns per thread, or one), "y_prefetch" (FP32 y passes with
 * column pairs as persistent blocks that double-buffer their tiles with
 * asynchronous copies: 0 neither, 1 the inverse pass (default), 2 both),
 * "overlap" (0/1: the k^2 half of the z inverse pass and the inverse y
 * transforms of its three fields on a second stream of the handle,
 * concurrently with the curl half and the y transforms of u),
 * "slab_pipe" (0/1: the y inverse, x and y passes over two halves of the
 * z-planes on two streams, the second half's y inverse after the first's),
 * "zf_pipe" (0/1: the z forward pass persistent, each thread copying the next
 * tile's inputs into its own shared slots once its epilogue is done), "fuse_stage" (0/1: the first nonlinear
 * term's z forward pass and the second term's z inverse pass as one kernel that
 * keeps the stage value c on chip, or two passes with c in HBM), "z_split" (z inverse
 * pass: 0 = one three-region kernel; 1 = w = k^2 a in its own one-region kernel;
 * 2 = one one-region kernel that reads the input columns again per output line;
 * 3 = the three-region kernel made persistent, each tile's inputs copied
 * asynchronously while the previous tile is transformed), "z_cluster" (mixed
 * form, 0/1: the z forward pass on thread-block cluster pairs, each CTA
 * holding half of a tile's z-rows and the pair's first radix-2 stage read
 * across them; the default for z columns of 1024 points or more), "z_tma" (mixed
 * form, bits: the z passes' tiles loaded by TMA, one thread issuing the tensor
 * copies of the three fields with an mbarrier each; 1 the z forward pass, 2
 * the z inverse pass; both the default for z columns of 256 and 512 points;
 * 4, with 2, the z inverse pass's six outputs written by tensor stores, the
 * default for z columns of 256 points). */
int gt_set_tuning(gt_handle* h, const char* key, int32_t value);
/* The current value of one gt_set_tuning knob (the per-grid default until
 * it is set). */
int gt_get_tuning(gt_handle* h, const char* key, int32_t* value);

/* Allocation-free kinetic energy, for callers that cannot allocate device
 * memory: a Fortran driver whose device arrays belong to another runtime (an
 * OpenACC data region, a pooled allocator holding the HBM) and that must not
 * call cudaMalloc/cudaFree in its time loop.  This entry point has no
 * counterpart in the reference.  bx, by, bz are the caller's DEVICE arrays
 * in the host layout above (FP64, [NZ][NY][NX/2+1][2]); energy_out is a
 * caller DEVICE array of 3 doubles that receives E_x, E_y, E_z of
 * gt_energy (same definition, FP64, fixed-order reduction), written on
 * `stream` (a cudaStream_t; NULL = the legacy default stream).  Scratch is a
 * fixed 6 MiB array inside the library (one partial per (y,z) row), held by
 * every GPU that loads the library until the process exits; grids with
 * NY*NZ > 262144 rows are rejected with GT_EINVAL.  The first call on a
 * device looks up that array's device address (cudaGetSymbolAddress, with
 * that device current), so make the first call before any stream capture;
 * the lookup is kept per device and CUDA context and repeated after the
 * context changes (after cudaDeviceReset the next call looks it up again and
 * should likewise come before any capture).
 * All calls on a device share the array: calls that overlap on the GPU race
 * and must be serialised by the caller. */
int gt_energy_noalloc(const double* bx, const double* by, const double* bz, int32_t nx,
                      int32_t ny, int32_t nz, double xlx, double xly, double xlz,
                      double* energy_out, void* stream);

/* ---- differentiation (no reference counterpart) ----------------------------
 * Tangent-linear and adjoint of one RK2 step at the current state (which is
 * left unchanged), for spectral perturbations / adjoint fields in the host
 * layout.  Adjoints are taken under <x, y> = sum over stored modes of
 * w Re(conj(x) y), w = 1 on the kx = 0 and kx = NX/2 planes and 2 elsewhere
 * (the full-spectrum inner product of real fields).  The forcing is additive
 * and state-independent, so it has no tangent. */
int gt_tl_step(gt_handle* h, const double* dbx, const double* dby, const double* dbz,
               double* ox, double* oy, double* oz);
int gt_adj_step(gt_handle* h, const double* lx, const double* ly, const double* lz,
                double* ox, double* oy, double* oz);
/* J = sum over stored modes with |k| >= kmin of fac |(curl b)_k|^2 (the
 * kinetic energy of those shells, fac as in glob). */
int gt_objective(gt_handle* h, double kmin, double* J);
/* Gradient of J after nsteps RK2 steps from the current state, with the
 * forcing realisation drawn from `seed` (not advanced), by a checkpointed
 * adjoint sweep (states stored every checkpoint_every steps and recomputed
 * per segment).  Writes J and dJ/db0 (so that dJ = <g, db0>); the state is
 * restored to its initial value. */
int gt_gradient(gt_handle* h, int32_t nsteps, int32_t seed, int32_t checkpoint_every, double kmin,
                double* J, double* gx, double* gy, double* gz);

/* Launch-shape autotuner: times whole RK2 steps (CUDA events) over the
 * gt_set_tuning knobs by coordinate descent on a copy of the current state,
 * keeps the fastest, and appends it to the JSON-lines cache at cache_path
 * (NULL: no cache), keyed by grid, precision, pruning and GPU name; a cached
 * choice is applied without timing.  *best_ms (may be NULL) gets the step
 * time, or -1 when the cache supplied the choice. */
int gt_autotune(gt_handle* h, const char* cache_path, double* best_ms);

/* ---- ensemble (no reference counterpart: the reference runs one field) ---- */
typedef struct gt_ensemble gt_ensemble;
/* n independent members (grids, physics and precision may differ; all on
 * members[0].device), each with the state and step of a gt_handle. */
int gt_ensemble_create(int32_t n, const gt_params* members, gt_ensemble** out);
int gt_ensemble_destroy(gt_ensemble* e);
int gt_ensemble_set_state(gt_ensemble* e, int32_t member, const double* bx, const double* by,
                          const double* bz);
int gt_ensemble_get_state(gt_ensemble* e, int32_t member, double* bx, double* by, double* bz);
/* nsteps RK2 steps of every member; seeds[n] are the members' forcing seeds
 * (advanced).  The forcing is drawn on the host in chunks of 64 steps.
 * graph = 1: one captured CUDA graph launch per chunk advances every member
 * by 64 steps (each class's batched launches, or a lone member's kernels, on
 * their own stream, joined at the end of the chunk; a shorter last chunk is
 * launched directly); graph = 0: the same launches issued directly. */
int gt_ensemble_step(gt_ensemble* e, int32_t nsteps, int32_t* seeds, int32_t graph);
/* Total kinetic energy of each member (n values). */
int gt_ensemble_energy(gt_ensemble* e, double* energy);
/* gt_autotune once per distinct (grid, precision) class, applied to all its members. */
int gt_ensemble_autotune(gt_ensemble* e, const char* cache_path);
/* Batched launches (on by default): members of one grid class (same grid, box,
 * precision and truncation; two or more members) keep their fields in one
 * device slab and every pass of the step runs as one launch for the whole
 * class, each member with its own integrating factor, Omega, dt and forcing;
 * classes and lone members run concurrently.  Off: each member's kernels are
 * launched on their own.  Results are the same either way. */
int gt_ensemble_set_batching(gt_ensemble* e, int32_t enable);
/* *nclasses = number of grid classes; class_of[i] (n values, may be NULL) =
 * member i's class, or -1 for a member that runs alone. */
int gt_ensemble_info(gt_ensemble* e, int32_t* nclasses, int32_t* class_of);

/* Exercises the bounded-wait failure path of the device waits without a
 * fault: a kernel waits on an mbarrier that nothing completes, gives up after a
 * few thousand polls and sets the handle's error flag.  Returns GT_ETIMEOUT
 * (and clears the flag); the handle stays usable.  No reference counterpart. */
int gt_selftest_wait_timeout(gt_handle* h);

/* Measures this GPU's ALU issue rates in G thread-instructions per second:
 * rates[0] DFMA, [1] DADD, [2] FFMA, [3] FADD (independent chains, 8 blocks of
 * 256 threads per SM).  The FP64 form of the step is FP64-ALU bound; these are
 * its roofline denominators.  No reference counterpart. */
int gt_probe_alu(int32_t device, double* rates);

/* Measures the DRAM rate that each pass's access pattern allows: copy kernels
 * that move exactly the algorithmic bytes of the z inverse, y inverse, x, y
 * forward and z forward passes of the handle's grid (the truncation-pruned
 * layout) with the passes' tile shapes and none of their arithmetic.  ms[0..4]
 * receive the milliseconds per launch, in that order; a pass's rate divided by
 * its pattern's rate says how far the pass is from the memory system's limit
 * for that pattern.  Overwrites the handle's work and stage buffers (not the
 * state).  GT_EINVAL when the pruned passes are not in use (untruncated or off
 * the kept set).  No reference counterpart. */
int gt_probe_patterns(gt_handle* h, double* ms);

/* ---- introspection ------------------------------------------------------- */
const char* gt_strerror(int code);
/* Text of the last CUDA failure seen on the calling thread ("" if none). */
const char* gt_last_error(void);
/* The cudaStream_t the handle launches on (for event timing by the caller). */
int gt_get_stream(gt_handle* h, void** stream);
/* Number of kernels this handle has launched since creation. */
int gt_launch_count(gt_handle* h, int64_t* count);
/* Per-kernel timing: while enabled, each launch is bracketed by CUDA events
 * on the handle's stream.  gt_profile_read returns, for up to cap kernel
 * kinds, a name, the number of launches and the summed milliseconds, and
 * resets the counters. */
int gt_profile_enable(gt_handle* h, int32_t on);
int gt_profile_read(gt_handle* h, int32_t cap, char* names /* cap x 32 bytes */,
                    int64_t* launches, double* ms, int32_t* nkinds);

#ifdef __cplusplus
}
#endif
#endif /* GTURBO_GB_H */
