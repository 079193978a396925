"""Host-side mirror of the reference's time-step interface over the C-ABI.

The names follow the reference's subroutines: ``step`` is the body of the
time loop (main.f90:121-150), ``nlt`` the nonlinear term (nlt.f90), ``glob`` /
``spectrum`` / ``fluxes`` the diagnostics (diagnostics.f90), ``fft_dir`` /
``fft_inv`` the transforms (fft_dir.f90, fft_inv.f90), ``rann`` the RNG
(forcing_3d3c.f90:82-93), ``read_params`` the params.dat reader
(inieuler.f90:14-20).  Spectral arrays are complex128[NZ, NY, NX//2+1] in C
order, the byte layout of the reference's complex*16 (NX/2+1, NY, NZ).

Every compute call runs on the GPU through ``libgturbo_gb.so``; there is no
CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import GtDiag, GtParams, check, load

_FORCING = {"none": _lib.GT_FORCING_NONE, "3d3c": _lib.GT_FORCING_3D3C, "2d2c": _lib.GT_FORCING_2D2C}
_DT2 = {"as_built": _lib.GT_DT2_AS_BUILT, "rk2": _lib.GT_DT2_RK2}
_PREC = {"fp64": _lib.GT_PREC_FP64, "mixed": _lib.GT_PREC_MIXED}


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_params(nx: int = 64, ny: int | None = None, nz: int | None = None, *, precision="fp64",
                forcing="3d3c", dt2_mode="rk2", device: int = 0, **physics) -> GtParams:
    """A parameter block: the params.dat defaults of a 2 pi box overridden by
    keyword arguments (xlx, xly, xlz, nu, alpnu, mu, alpmu, dt, omega, rtrunc,
    truncate, famp, k1f, k2f)."""
    lib = load()
    p = GtParams()
    check(lib.gt_params_default(C.byref(p)), "gt_params_default")
    p.nx, p.ny, p.nz = nx, ny or nx, nz or nx
    p.precision = _PREC[precision]
    p.forcing = _FORCING[forcing]
    p.dt2_mode = _DT2[dt2_mode]
    p.device = device
    for k, v in physics.items():
        if not hasattr(p, k):
            raise TypeError(f"unknown parameter {k!r}")
        setattr(p, k, v)
    return p


def read_params(path: str, base: GtParams | None = None) -> GtParams:
    """params.dat (inieuler.f90:14-20) into a parameter block."""
    lib = load()
    p = base if base is not None else make_params()
    check(lib.gt_params_read(str(path).encode(), C.byref(p)), "gt_params_read")
    return p


def memory_estimate(p: GtParams) -> int:
    """Device bytes gt_create allocates for p."""
    n = C.c_size_t()
    check(load().gt_memory_estimate(C.byref(p), C.byref(n)), "gt_memory_estimate")
    return n.value


def set_memory_budget(nbytes: int) -> None:
    """Process-wide cap on one handle's device bytes (0 = none): gt_create
    returns GT_ENOMEM above it, decided on the host before any CUDA call."""
    check(load().gt_set_memory_budget(C.c_uint64(int(nbytes))), "gt_set_memory_budget")


def memory_budget() -> int:
    v = C.c_uint64()
    check(load().gt_get_memory_budget(C.byref(v)), "gt_get_memory_budget")
    return v.value


def probe_alu(device: int = 0) -> dict:
    """This GPU's ALU issue rates (gt_probe_alu), G thread-instructions/s."""
    lib = load()
    r = np.zeros(4)
    check(lib.gt_probe_alu(int(device), _dp(r)), "gt_probe_alu")
    return {"dfma": float(r[0]), "dadd": float(r[1]), "ffma": float(r[2]), "fadd": float(r[3])}


def rann(seed: int, n: int) -> tuple[np.ndarray, int]:
    """n draws of the reference RNG from state ``seed``; returns (values, seed)."""
    lib = load()
    s = C.c_int32(seed)
    out = np.zeros(n, np.float32)
    check(lib.gt_rann(C.byref(s), n, out.ctypes.data_as(C.POINTER(C.c_float))), "gt_rann")
    return out, s.value


@dataclass
class ForcedModes:
    ix: np.ndarray
    iy: np.ndarray
    iz: np.ndarray
    ff: np.ndarray
    inpe: float
    inpz: float

    @property
    def nf(self) -> int:
        return len(self.ix)


def forced_modes(p: GtParams) -> ForcedModes:
    """The forced-mode list in the reference's order (iniforcing_*.f90)."""
    lib = load()
    n = _lib.GT_NFORC
    ix, iy, iz = (np.zeros(n, np.int32) for _ in range(3))
    ff = np.zeros(n)
    nf = C.c_int32()
    inpe, inpz = C.c_double(), C.c_double()
    ip = C.POINTER(C.c_int32)
    check(lib.gt_forced_modes(C.byref(p), C.byref(nf), ix.ctypes.data_as(ip), iy.ctypes.data_as(ip),
                              iz.ctypes.data_as(ip), _dp(ff), C.byref(inpe), C.byref(inpz)),
          "gt_forced_modes")
    m = nf.value
    return ForcedModes(ix[:m].copy(), iy[:m].copy(), iz[:m].copy(), ff[:m].copy(), inpe.value, inpz.value)


def forcing_increments(p: GtParams, seed: int):
    """One step's forcing adds in the reference's order (forcing_3d3c.f90 /
    forcing_2d2c.f90): returns (ix, iy, iz, dF[n, 6], new_seed)."""
    lib = load()
    cap = 2 * _lib.GT_NFORC
    ix, iy, iz = (np.zeros(cap, np.int32) for _ in range(3))
    dF = np.zeros((cap, 6))
    s = C.c_int32(seed)
    n = C.c_int32()
    ip = C.POINTER(C.c_int32)
    check(lib.gt_forcing_increments(C.byref(p), C.byref(s), cap, C.byref(n), ix.ctypes.data_as(ip),
                                    iy.ctypes.data_as(ip), iz.ctypes.data_as(ip), _dp(dF)),
          "gt_forcing_increments")
    m = n.value
    return ix[:m].copy(), iy[:m].copy(), iz[:m].copy(), dF[:m].copy(), s.value


def init_noise(p: GtParams, seed: int):
    """The reference's fresh-start noise (trunc.f90:75-93): returns the three
    physical components (double[NZ][NY][NX], sqrt(dt) (rann - 0.5) each) and
    the advanced seed; Simulation.set_state_physical turns them into the
    initial state (main.f90:91-106)."""
    lib = load()
    u = [np.zeros((p.nz, p.ny, p.nx)) for _ in range(3)]
    s = C.c_int32(seed)
    check(lib.gt_init_noise(C.byref(p), C.byref(s), _dp(u[0]), _dp(u[1]), _dp(u[2])), "gt_init_noise")
    return u, s.value


def forcing_amplitude(injection: float, p: GtParams) -> float:
    """famp giving the mean energy input nf famp^2 = injection (iniforcing_3d3c.f90:39)."""
    nf = forced_modes(p).nf
    return math.sqrt(injection / nf) if nf else 0.0


def read_seed(path: str) -> int:
    s = C.c_int32()
    check(load().gt_seed_read(str(path).encode(), C.byref(s)), "gt_seed_read")
    return s.value


def write_seed(path: str, seed: int) -> None:
    check(load().gt_seed_write(str(path).encode(), seed), "gt_seed_write")


def read_frame(path: str) -> tuple[int, float]:
    """curframe.dat: (ifr, t) a continuation starts from (main.f90:37-39)."""
    f, t = C.c_int32(), C.c_double()
    check(load().gt_frame_read(str(path).encode(), C.byref(f), C.byref(t)), "gt_frame_read")
    return f.value, t.value


def write_frame(path: str, ifr: int, t: float) -> None:
    check(load().gt_frame_write(str(path).encode(), ifr, t), "gt_frame_write")


def read_field(path: str, nx: int, ny: int, nz: int) -> np.ndarray:
    """One float32 velocity component, fields/u?.NNN (read.f90:12-22)."""
    out = np.zeros((nz, ny, nx), np.float32)
    check(load().gt_field_read_f32(str(path).encode(), nx, ny, nz,
                                   out.ctypes.data_as(C.POINTER(C.c_float))), "gt_field_read_f32")
    return out


def write_field(path: str, u: np.ndarray) -> None:
    """One float32 velocity component as written by writef (write.f90:12-22)."""
    nz, ny, nx = u.shape
    a = np.ascontiguousarray(u, np.float32)
    check(load().gt_field_write_f32(str(path).encode(), nx, ny, nz,
                                    a.ctypes.data_as(C.POINTER(C.c_float))), "gt_field_write_f32")


class Simulation:
    """One device-resident state b (the vector potential) and its time step."""

    def __init__(self, params: GtParams | None = None, **kw):
        self.lib = load()
        self.params = params if params is not None else make_params(**kw)
        h = C.c_void_p()
        check(self.lib.gt_create(C.byref(self.params), C.byref(h)), "gt_create")
        self.h = h
        p = self.params
        self.shape = (p.nz, p.ny, p.nx // 2 + 1)
        self.rshape = (p.nz, p.ny, p.nx)

    # -- life cycle ---------------------------------------------------------
    def close(self):
        if self.h:
            self.lib.gt_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state -------------------------------------------------------------
    def _spec_in(self, a):
        a = np.ascontiguousarray(a, np.complex128)
        if a.shape != self.shape:
            raise ValueError(f"expected a {self.shape} spectral field, got {a.shape}")
        return a

    def set_state(self, b):
        b = [self._spec_in(x) for x in b]
        check(self.lib.gt_set_state(self.h, *(_dp(x.view(np.float64)) for x in b)), "gt_set_state")

    def get_state(self):
        out = [np.empty(self.shape, np.complex128) for _ in range(3)]
        check(self.lib.gt_get_state(self.h, *(_dp(x.view(np.float64)) for x in out)), "gt_get_state")
        return out

    # -- the time step (main.f90:121-150) ------------------------------------
    def step(self, nsteps: int = 1, seed: int | None = None) -> int | None:
        """Advances nsteps RK2 steps; returns the advanced forcing seed."""
        if seed is None:
            check(self.lib.gt_rk2_step(self.h, nsteps, None), "gt_rk2_step")
            return None
        s = C.c_int32(seed)
        check(self.lib.gt_rk2_step(self.h, nsteps, C.byref(s)), "gt_rk2_step")
        return s.value

    def step_coeffs(self, ix, iy, iz, dF):
        """One RK2 step whose forcing is the caller's list of increments:
        dF[e] = [Re bx, Im bx, Re by, Im by, Re bz, Im bz]."""
        ix, iy, iz = (np.ascontiguousarray(v, np.int32) for v in (ix, iy, iz))
        dF = np.ascontiguousarray(dF, np.float64).reshape(-1, 6)
        ip = C.POINTER(C.c_int32)
        check(self.lib.gt_rk2_step_coeffs(self.h, len(ix), ix.ctypes.data_as(ip), iy.ctypes.data_as(ip),
                                          iz.ctypes.data_as(ip), _dp(dF)), "gt_rk2_step_coeffs")

    def nlt(self, a):
        """N = nlt(a) with the current state as the Coriolis source (nlt.f90)."""
        a = [self._spec_in(x) for x in a]
        out = [np.empty(self.shape, np.complex128) for _ in range(3)]
        check(self.lib.gt_nonlinear(self.h, *(_dp(x.view(np.float64)) for x in a),
                                    *(_dp(x.view(np.float64)) for x in out)), "gt_nonlinear")
        return out

    # -- diagnostics (diagnostics.f90) ---------------------------------------
    def diagnostics(self, flux: bool = True) -> dict:
        nbin = self.params.nx // 2
        d = GtDiag()
        ek, ek2d = np.zeros(nbin), np.zeros(nbin)
        fl = np.zeros(nbin) if flux else None
        check(self.lib.gt_diagnostics(self.h, C.byref(d), _dp(ek), _dp(ek2d),
                                      _dp(fl) if flux else None), "gt_diagnostics")
        return {
            "energy": np.array(d.energy[:]), "enstrophy": np.array(d.enstrophy[:]),
            "helicity": d.helicity, "inpe": d.inpe, "inpz": d.inpz, "nonfinite": d.nonfinite,
            "spectrum": ek, "spectrum2d": ek2d, "flux": fl,
        }

    def glob(self) -> dict:
        d = self.diagnostics(flux=False)
        return {"energy": d["energy"], "enstrophy": d["enstrophy"]}

    def energy(self) -> float:
        """Total kinetic energy (sum of glob's three energy terms)."""
        e = np.zeros(3)
        check(self.lib.gt_energy(self.h, _dp(e)), "gt_energy")
        return float(e.sum())

    def spectrum(self):
        d = self.diagnostics(flux=False)
        return d["spectrum"], d["spectrum2d"]

    def fluxes(self):
        return self.diagnostics(flux=True)["flux"]

    def check_finite(self) -> int:
        return self.lib.gt_check_finite(self.h)

    def selftest_wait_timeout(self) -> int:
        """Runs the bounded-wait self-test; returns its status (GT_ETIMEOUT = -7
        when the wait ran out as it should)."""
        return self.lib.gt_selftest_wait_timeout(self.h)

    def set_tuning(self, key: str, value: int) -> None:
        check(self.lib.gt_set_tuning(self.h, key.encode(), int(value)), f"gt_set_tuning({key})")

    def get_tuning(self, key: str) -> int:
        v = C.c_int32()
        check(self.lib.gt_get_tuning(self.h, key.encode(), C.byref(v)), f"gt_get_tuning({key})")
        return v.value

    PATTERN_PASSES = ("zinv_curl", "yinv", "xcross", "yfwd", "zfwd_epilogue")

    def probe_patterns(self) -> dict:
        """Milliseconds per launch of copy kernels with each pass's access
        pattern and algorithmic bytes (gt_probe_patterns), keyed like the
        bench's pass names.  Overwrites the work and stage buffers, not the state."""
        r = np.zeros(5)
        check(self.lib.gt_probe_patterns(self.h, _dp(r)), "gt_probe_patterns")
        return dict(zip(self.PATTERN_PASSES, (float(x) for x in r)))

    def set_pruning(self, enable: bool) -> None:
        check(self.lib.gt_set_pruning(self.h, 1 if enable else 0), "gt_set_pruning")

    @property
    def pruning_active(self) -> bool:
        a = C.c_int32()
        check(self.lib.gt_pruning_active(self.h, C.byref(a)), "gt_pruning_active")
        return bool(a.value)

    # -- transforms and the initial / output paths ---------------------------
    def fft_dir(self, x):
        x = np.ascontiguousarray(x, np.float64)
        if x.shape != self.rshape:
            raise ValueError(f"expected a {self.rshape} real field")
        out = np.empty(self.shape, np.complex128)
        check(self.lib.gt_fft_dir(self.h, _dp(x), _dp(out.view(np.float64))), "gt_fft_dir")
        return out

    def fft_inv(self, z):
        z = self._spec_in(z)
        out = np.empty(self.rshape, np.float64)
        check(self.lib.gt_fft_inv(self.h, _dp(z.view(np.float64)), _dp(out)), "gt_fft_inv")
        return out

    def velocity(self):
        out = [np.empty(self.rshape, np.float64) for _ in range(3)]
        check(self.lib.gt_velocity(self.h, *(_dp(x) for x in out)), "gt_velocity")
        return out

    def set_state_physical(self, u) -> float:
        u = [np.ascontiguousarray(x, np.float64) for x in u]
        cc = C.c_double()
        check(self.lib.gt_set_state_physical(self.h, *(_dp(x) for x in u), C.byref(cc)),
              "gt_set_state_physical")
        return cc.value

    # -- differentiation ----------------------------------------------------
    def tl_step(self, db):
        """Tangent-linear RK2 step at the current state."""
        db = [self._spec_in(x) for x in db]
        out = [np.empty(self.shape, np.complex128) for _ in range(3)]
        check(self.lib.gt_tl_step(self.h, *(_dp(x.view(np.float64)) for x in db),
                                  *(_dp(x.view(np.float64)) for x in out)), "gt_tl_step")
        return out

    def adj_step(self, lam):
        """Adjoint RK2 step at the current state."""
        lam = [self._spec_in(x) for x in lam]
        out = [np.empty(self.shape, np.complex128) for _ in range(3)]
        check(self.lib.gt_adj_step(self.h, *(_dp(x.view(np.float64)) for x in lam),
                                   *(_dp(x.view(np.float64)) for x in out)), "gt_adj_step")
        return out

    def objective(self, kmin: float) -> float:
        j = C.c_double()
        check(self.lib.gt_objective(self.h, kmin, C.byref(j)), "gt_objective")
        return j.value

    def gradient(self, nsteps: int, seed: int, checkpoint_every: int, kmin: float):
        """(J, dJ/db0) of the shell energy after nsteps steps (gt_gradient)."""
        j = C.c_double()
        out = [np.empty(self.shape, np.complex128) for _ in range(3)]
        check(self.lib.gt_gradient(self.h, nsteps, seed, checkpoint_every, kmin, C.byref(j),
                                   *(_dp(x.view(np.float64)) for x in out)), "gt_gradient")
        return j.value, out

    # -- introspection -----------------------------------------------------
    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(self.lib.gt_get_stream(self.h, C.byref(s)), "gt_get_stream")
        return s.value or 0

    def launch_count(self) -> int:
        n = C.c_int64()
        check(self.lib.gt_launch_count(self.h, C.byref(n)), "gt_launch_count")
        return n.value

    def profile(self, on: bool = True):
        check(self.lib.gt_profile_enable(self.h, 1 if on else 0), "gt_profile_enable")

    def profile_read(self) -> dict:
        cap = 32
        names = C.create_string_buffer(32 * cap)
        launches = (C.c_int64 * cap)()
        ms = (C.c_double * cap)()
        n = C.c_int32()
        check(self.lib.gt_profile_read(self.h, cap, names, launches, ms, C.byref(n)), "gt_profile_read")
        out = {}
        raw = names.raw
        for i in range(n.value):
            nm = raw[32 * i:32 * i + 32].split(b"\0", 1)[0].decode()
            out[nm] = (int(launches[i]), float(ms[i]))
        return out


def autotune(sim: "Simulation", cache_path: str | None = None) -> float:
    """Chooses the fastest launch shapes for sim's grid and precision
    (gt_autotune); returns the step time in ms, or -1 if taken from the cache."""
    ms = C.c_double()
    check(sim.lib.gt_autotune(sim.h, cache_path.encode() if cache_path else None, C.byref(ms)),
          "gt_autotune")
    return ms.value


class Ensemble:
    """Independent members advanced together (gt_ensemble_*): members of one
    grid class share one launch per pass; in graph mode one captured CUDA
    graph launch advances every member by 64 steps."""

    def __init__(self, params: list):
        self.lib = load()
        n = len(params)
        arr = (GtParams * n)(*params)
        h = C.c_void_p()
        check(self.lib.gt_ensemble_create(n, arr, C.byref(h)), "gt_ensemble_create")
        self.h = h
        self.n = n
        self.shapes = [(p.nz, p.ny, p.nx // 2 + 1) for p in params]

    def close(self):
        if self.h:
            self.lib.gt_ensemble_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, i: int, b):
        b = [np.ascontiguousarray(x, np.complex128) for x in b]
        if b[0].shape != self.shapes[i]:
            raise ValueError("shape mismatch")
        check(self.lib.gt_ensemble_set_state(self.h, i, *(_dp(x.view(np.float64)) for x in b)),
              "gt_ensemble_set_state")

    def get_state(self, i: int):
        out = [np.empty(self.shapes[i], np.complex128) for _ in range(3)]
        check(self.lib.gt_ensemble_get_state(self.h, i, *(_dp(x.view(np.float64)) for x in out)),
              "gt_ensemble_get_state")
        return out

    def step(self, nsteps: int, seeds, graph: bool = True) -> np.ndarray:
        s = np.ascontiguousarray(seeds, np.int32).copy()
        check(self.lib.gt_ensemble_step(self.h, nsteps, s.ctypes.data_as(C.POINTER(C.c_int32)),
                                        1 if graph else 0), "gt_ensemble_step")
        return s

    def energy(self) -> np.ndarray:
        e = np.zeros(self.n)
        check(self.lib.gt_ensemble_energy(self.h, _dp(e)), "gt_ensemble_energy")
        return e

    def autotune(self, cache_path: str | None = None):
        check(self.lib.gt_ensemble_autotune(self.h, cache_path.encode() if cache_path else None),
              "gt_ensemble_autotune")

    def set_batching(self, enable: bool) -> None:
        """One launch per pass for each grid class (on, the default) or per member."""
        check(self.lib.gt_ensemble_set_batching(self.h, 1 if enable else 0), "gt_ensemble_set_batching")

    def classes(self) -> list:
        """Each member's grid class (-1: runs alone)."""
        n = C.c_int32()
        cls = np.zeros(self.n, np.int32)
        check(self.lib.gt_ensemble_info(self.h, C.byref(n), cls.ctypes.data_as(C.POINTER(C.c_int32))),
              "gt_ensemble_info")
        return [int(x) for x in cls]
