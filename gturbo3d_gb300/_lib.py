"""ctypes binding of ``libgturbo_gb.so`` (the C-ABI in include/gturbo_gb.h).

Loading fails loudly: there is no CPU fallback for any compute entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libgturbo_gb.so"

GT_OK = 0
GT_EINVAL = -1
GT_ENOMEM = -2
GT_ECUDA = -3
GT_ENFORC = -4
GT_ENONFINITE = -5
GT_EIO = -6
GT_ETIMEOUT = -7

GT_FORCING_NONE, GT_FORCING_3D3C, GT_FORCING_2D2C = 0, 1, 2
GT_DT2_AS_BUILT, GT_DT2_RK2 = 0, 1
GT_PREC_FP64, GT_PREC_MIXED = 0, 1
GT_NFORC = 2048


class GtParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("xlx", C.c_double), ("xly", C.c_double), ("xlz", C.c_double),
        ("nu", C.c_double), ("alpnu", C.c_double), ("mu", C.c_double), ("alpmu", C.c_double),
        ("dt", C.c_double), ("omega", C.c_double),
        ("rtrunc", C.c_double), ("truncate", C.c_int32),
        ("famp", C.c_double), ("k1f", C.c_double), ("k2f", C.c_double),
        ("forcing", C.c_int32), ("dt2_mode", C.c_int32), ("precision", C.c_int32),
        ("device", C.c_int32),
    ]


class GtDiag(C.Structure):
    _fields_ = [
        ("energy", C.c_double * 9), ("enstrophy", C.c_double * 9), ("helicity", C.c_double),
        ("inpe", C.c_double), ("inpz", C.c_double), ("nonfinite", C.c_int64),
    ]


_P = C.POINTER
_dp = _P(C.c_double)
_ip = _P(C.c_int32)
_vp = C.c_void_p

# name -> (restype, argtypes); every symbol include/gturbo_gb.h declares
SIGNATURES = {
    "gt_params_default": (C.c_int, [_P(GtParams)]),
    "gt_params_validate": (C.c_int, [_P(GtParams)]),
    "gt_params_read": (C.c_int, [C.c_char_p, _P(GtParams)]),
    "gt_memory_estimate": (C.c_int, [_P(GtParams), _P(C.c_size_t)]),
    "gt_set_memory_budget": (C.c_int, [C.c_uint64]),
    "gt_get_memory_budget": (C.c_int, [_P(C.c_uint64)]),
    "gt_rann": (C.c_int, [_ip, C.c_int32, _P(C.c_float)]),
    "gt_forced_modes": (C.c_int, [_P(GtParams), _ip, _ip, _ip, _ip, _dp, _dp, _dp]),
    "gt_forcing_increments": (C.c_int, [_P(GtParams), _ip, C.c_int32, _ip, _ip, _ip, _ip, _dp]),
    "gt_init_noise": (C.c_int, [_P(GtParams), _ip, _dp, _dp, _dp]),
    "gt_seed_read": (C.c_int, [C.c_char_p, _ip]),
    "gt_seed_write": (C.c_int, [C.c_char_p, C.c_int32]),
    "gt_frame_read": (C.c_int, [C.c_char_p, _ip, _dp]),
    "gt_frame_write": (C.c_int, [C.c_char_p, C.c_int32, C.c_double]),
    "gt_field_read_f32": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, _P(C.c_float)]),
    "gt_field_write_f32": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, _P(C.c_float)]),
    "gt_create": (C.c_int, [_P(GtParams), _P(_vp)]),
    "gt_destroy": (C.c_int, [_vp]),
    "gt_set_state": (C.c_int, [_vp, _dp, _dp, _dp]),
    "gt_get_state": (C.c_int, [_vp, _dp, _dp, _dp]),
    "gt_rk2_step": (C.c_int, [_vp, C.c_int32, _ip]),
    "gt_rk2_step_coeffs": (C.c_int, [_vp, C.c_int32, _ip, _ip, _ip, _dp]),
    "gt_nonlinear": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "gt_diagnostics": (C.c_int, [_vp, _P(GtDiag), _dp, _dp, _dp]),
    "gt_energy": (C.c_int, [_vp, _dp]),
    "gt_energy_noalloc": (C.c_int, [_vp, _vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                                    C.c_double, C.c_double, _vp, _vp]),
    "gt_fft_dir": (C.c_int, [_vp, _dp, _dp]),
    "gt_fft_inv": (C.c_int, [_vp, _dp, _dp]),
    "gt_velocity": (C.c_int, [_vp, _dp, _dp, _dp]),
    "gt_set_state_physical": (C.c_int, [_vp, _dp, _dp, _dp, _dp]),
    "gt_check_finite": (C.c_int, [_vp]),
    "gt_set_pruning": (C.c_int, [_vp, C.c_int32]),
    "gt_pruning_active": (C.c_int, [_vp, _ip]),
    "gt_selftest_wait_timeout": (C.c_int, [_vp]),
    "gt_probe_alu": (C.c_int, [C.c_int32, _dp]),
    "gt_probe_patterns": (C.c_int, [_vp, _dp]),
    "gt_set_tuning": (C.c_int, [_vp, C.c_char_p, C.c_int32]),
    "gt_get_tuning": (C.c_int, [_vp, C.c_char_p, _ip]),
    "gt_autotune": (C.c_int, [_vp, C.c_char_p, _dp]),
    "gt_tl_step": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "gt_adj_step": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "gt_objective": (C.c_int, [_vp, C.c_double, _dp]),
    "gt_gradient": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int32, C.c_double, _dp, _dp, _dp, _dp]),
    "gt_ensemble_create": (C.c_int, [C.c_int32, _P(GtParams), _P(_vp)]),
    "gt_ensemble_destroy": (C.c_int, [_vp]),
    "gt_ensemble_set_state": (C.c_int, [_vp, C.c_int32, _dp, _dp, _dp]),
    "gt_ensemble_get_state": (C.c_int, [_vp, C.c_int32, _dp, _dp, _dp]),
    "gt_ensemble_step": (C.c_int, [_vp, C.c_int32, _ip, C.c_int32]),
    "gt_ensemble_energy": (C.c_int, [_vp, _dp]),
    "gt_ensemble_autotune": (C.c_int, [_vp, C.c_char_p]),
    "gt_ensemble_set_batching": (C.c_int, [_vp, C.c_int32]),
    "gt_ensemble_info": (C.c_int, [_vp, _ip, _ip]),
    "gt_strerror": (C.c_char_p, [C.c_int]),
    "gt_last_error": (C.c_char_p, []),
    "gt_get_stream": (C.c_int, [_vp, _P(_vp)]),
    "gt_launch_count": (C.c_int, [_vp, _P(C.c_int64)]),
    "gt_profile_enable": (C.c_int, [_vp, C.c_int32]),
    "gt_profile_read": (C.c_int, [_vp, C.c_int32, C.c_char_p, _P(C.c_int64), _dp, _ip]),
}

_lib = None


def load(path: Path | str | None = None):
    """Loads the library (once).  Raises if it is missing: build it with
    ``gturbo3d_gb300.build.build()``."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build the CUDA library first "
                          "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class GturboError(RuntimeError):
    def __init__(self, code: int, where: str):
        lib = load()
        msg = lib.gt_strerror(code).decode()
        detail = lib.gt_last_error().decode()
        super().__init__(f"{where}: status {code} ({msg}){': ' + detail if detail else ''}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != GT_OK:
        raise GturboError(code, where)
