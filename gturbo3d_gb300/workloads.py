"""Parameter sets of the synthetic benchmark configurations beyond the 512^3
roofline case, and the small host helpers they need (CFL time step, the
half-spectrum inner product, random directions).

* ``precision_params``: 256^3, nu = 5e-4, Omega = 10, dt = 2e-3, 2D2C forcing on
  2 <= |k_h| <= 3 (kz = 0 modes) at injection 0.1, seed 1, 200 steps; plain
  FP64 against mixed.
* ``ensemble_members``: 48 members at 64^3, 12 at 128^3 and 4 at 256^3, seeds
  100..163, Omega uniform in [1, 20] (drawn with the reference's 31-bit LCG
  from the member's seed), nu from k_max eta = 1.5 with the injection rate as
  the dissipation (eta = (nu^3 / eps)^(1/4), k_max = N/3 after 2/3
  truncation), dt from CFL 0.5 on the member's initial field, 3D3C forcing.
* ``adjoint_params``: 128^3, nu = 1e-3, Omega = 5, dt = 4e-3, 3D3C forcing
  realisation of seed 3, 200 steps, objective = kinetic energy of the shells
  |k| >= 20, checkpoints every 20 steps.

The initial fields are the seeded synthetic potentials of ``synth``.
"""
from __future__ import annotations

import math

import numpy as np

from .api import forcing_amplitude, make_params
from .synth import initial_potential, lcg_stream

INJECTION = 0.1


def cfl_dt(b, n: int, cfl: float = 0.5, xl: float = 2.0 * math.pi) -> float:
    """dt = cfl * dx / max(|u_x| + |u_y| + |u_z|) for the velocity u = curl b
    of a spectral vector potential b (complex[nz, ny, nx//2+1] each)."""
    import scipy.fft as sfft

    nz, ny, nh = b[0].shape
    nx = 2 * (nh - 1)
    kx = 2 * math.pi / xl * np.arange(nh)
    ky = 2 * math.pi / xl * np.fft.fftfreq(ny, 1.0 / ny)
    kz = 2 * math.pi / xl * np.fft.fftfreq(nz, 1.0 / nz)
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    ux = 1j * (KY * b[2] - KZ * b[1])
    uy = 1j * (KZ * b[0] - KX * b[2])
    uz = 1j * (KX * b[1] - KY * b[0])
    s = np.zeros((nz, ny, nx))
    for u in (ux, uy, uz):
        s += np.abs(sfft.irfftn(u, s=(nz, ny, nx), norm="forward"))
    return cfl * (xl / n) / float(s.max())


def kolmogorov_nu(n: int, eps: float = INJECTION, kmax_eta: float = 1.5) -> float:
    """nu with k_max eta = kmax_eta, k_max = n/3, eta = (nu^3/eps)^(1/4)."""
    eta = kmax_eta / (n / 3.0)
    return (eta ** 4 * eps) ** (1.0 / 3.0)


def ensemble_members():
    """The 64 members of the batched-ensemble configuration: dicts with grid
    size n, seed, omega, nu, dt and the initial potential b0."""
    sizes = [64] * 48 + [128] * 12 + [256] * 4
    out = []
    for i, n in enumerate(sizes):
        seed = 100 + i
        r, _ = lcg_stream(seed, 1)
        omega = 1.0 + 19.0 * float(r[0])
        b0 = initial_potential(n, n, n, seed)
        out.append({"n": n, "seed": seed, "omega": omega, "nu": kolmogorov_nu(n),
                    "dt": cfl_dt(b0, n), "b0": b0})
    return out


def ensemble_params(members, precision: str = "mixed"):
    ps = []
    for m in members:
        p = make_params(m["n"], precision=precision, forcing="3d3c", nu=m["nu"], omega=m["omega"], dt=m["dt"])
        p.famp = forcing_amplitude(INJECTION, p)
        ps.append(p)
    return ps


def precision_params(precision: str, n: int = 256):
    p = make_params(n, precision=precision, forcing="2d2c", nu=5e-4, omega=10.0, dt=2e-3)
    p.famp = forcing_amplitude(INJECTION, p)
    return p


def adjoint_params(precision: str, n: int = 128):
    p = make_params(n, precision=precision, forcing="3d3c", nu=1e-3, omega=5.0, dt=4e-3)
    p.famp = forcing_amplitude(INJECTION, p)
    return p


def spectral_inner(x, y) -> float:
    """<x, y> = sum over stored modes of w Re(conj(x) y), w = 1 on the kx = 0
    and kx = NX/2 planes and 2 elsewhere (the full-spectrum sum of real
    fields); the inner product under which gt_adj_step is the adjoint."""
    tot = 0.0
    for a, b in zip(x, y):
        p = (np.conj(a) * b).real
        tot += 2.0 * float(p.sum()) - float(p[..., 0].sum()) - float(p[..., -1].sum())
    return tot


def random_direction(n: int, seed: int, scale_to=None):
    """A seeded smooth random vector potential (the spectrum of a real
    field), optionally scaled to the norm of ``scale_to``."""
    d = initial_potential(n, n, n, seed)
    if scale_to is not None:
        f = math.sqrt(spectral_inner(scale_to, scale_to) / spectral_inner(d, d))
        d = [f * x for x in d]
    return d
