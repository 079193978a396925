"""Builds matching oracle / library configurations for the parity tests."""
import numpy as np


def configs(n, precision="fp64", forcing="3d3c", dt2_mode="rk2", **phys):
    """(library params, oracle params) for the same run."""
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Params
    nx, ny, nz = n if isinstance(n, tuple) else (n, n, n)
    gp = g.make_params(nx, ny, nz, precision=precision, forcing=forcing, dt2_mode=dt2_mode, **phys)
    op = Params(nx=nx, ny=ny, nz=nz, forcing=forcing, dt2_mode=dt2_mode, **phys)
    return gp, op


def initial(n, seed=0, **kw):
    from gturbo3d_gb300.synth import initial_potential
    nx, ny, nz = n if isinstance(n, tuple) else (n, n, n)
    return initial_potential(nx, ny, nz, seed, **kw)


def relerr(a, b):
    """sqrt(sum |a-b|^2 / sum |b|^2) over a list of arrays."""
    num = sum(float(np.sum(np.abs(np.asarray(x) - np.asarray(y)) ** 2)) for x, y in zip(a, b))
    den = sum(float(np.sum(np.abs(np.asarray(y)) ** 2)) for y in b)
    return np.sqrt(num / den) if den > 0 else np.sqrt(num)
