"""Seeded synthetic inputs: the initial vector potential and the forcing
amplitude for the benchmark and test configurations.

The reference starts either from a restart file or from zero plus real-space
noise (inieuler.f90:76-85); the benchmark configurations instead prescribe a
random-phase solenoidal field with E(k) ~ k^4 exp(-2 (k/k_p)^2) normalised to a
total energy E0.  This module generates that field on the host, deterministically
from a seed, with the reference's own 31-bit LCG (forcing_3d3c.f90:82-93) as the
source of randomness:

1. for every half-space mode, in memory order (z slowest, x fastest), draw six
   ``rann`` values r0..r5 and set u_c = (r_{2c} - 1/2) + i (r_{2c+1} - 1/2);
2. remove the k-parallel part (k = 0 set to zero);
3. scale each integer shell s = nint(|k|) so that its energy
   sum fac |u|^2 equals s^4 exp(-2 (s/k_p)^2);
4. make the field the transform of a real field (inverse then forward 3D FFT);
5. b = i k x u / k^2 (velocity -> vector potential, produ.f90:79-101), then the
   2/3 truncation (trunc.f90:10-28) when ``truncate`` is set;
6. rescale so that E = sum_k fac |curl b|^2 (the energy of diagnostics.f90:126-153)
   equals E0.

This is input synthesis, not the time-step path: it runs once before any step.
"""
from __future__ import annotations

import math

import numpy as np

_LCG_MUL = 69069
_LCG_MASK = 0x7FFFFFFF
PI_REF = 3.14159265358979323846


def lcg_stream(seed: int, n: int) -> tuple[np.ndarray, int]:
    """``n`` consecutive draws of rann (REAL*4(irand / (2^31-1)) after
    irand = (69069 irand + 1) mod 2^31) from state ``seed``.  Returns the float32
    values and the final state."""
    seed = int(seed) & 0xFFFFFFFF
    if n <= 0:
        return np.zeros(0, np.float32), seed & _LCG_MASK if seed else 0
    B = min(n, 8192)
    first = np.empty(B, dtype=np.uint64)
    x = seed
    for j in range(B):
        x = (_LCG_MUL * x + 1) & _LCG_MASK
        first[j] = x
    A, C = 1, 0
    for _ in range(B):
        A, C = (_LCG_MUL * A) & _LCG_MASK, (_LCG_MUL * C + 1) & _LCG_MASK
    nblk = (n + B - 1) // B
    out = np.empty(nblk * B, dtype=np.uint64)
    out[:B] = first
    A64, C64, M = np.uint64(A), np.uint64(C), np.uint64(_LCG_MASK)
    cur = first
    for m in range(1, nblk):
        cur = (A64 * cur + C64) & M
        out[m * B:(m + 1) * B] = cur
    out = out[:n]
    return (out.astype(np.float64) / float(_LCG_MASK)).astype(np.float32), int(out[-1])


def _wavenumbers(n: int, xl: float, half: bool):
    dk = 2.0 * PI_REF / xl
    if half:
        return np.arange(n // 2 + 1, dtype=np.float64) * dk
    k = np.arange(n, dtype=np.float64)
    k[k > n // 2] -= n
    return k * dk


def forcing_amplitude(injection: float, nf: int) -> float:
    """famp such that the mean energy input nf * famp^2 (iniforcing_3d3c.f90:39,
    with ff = 1/|k|) equals ``injection``."""
    return math.sqrt(injection / nf) if nf > 0 else 0.0


def initial_potential(nx: int, ny: int, nz: int, seed: int, e0: float = 0.5, kpeak: float = 3.0,
                      xl=(2.0 * PI_REF,) * 3, rtrunc: float = 0.6666666666666666667,
                      truncate: int = 1):
    """Returns [bx, by, bz], each complex128[nz, ny, nx//2+1] (the reference's
    complex*16 (NX/2+1, NY, NZ) layout)."""
    import scipy.fft as sfft

    nh = nx // 2 + 1
    kx = _wavenumbers(nx, xl[0], True)[None, None, :]
    ky = _wavenumbers(ny, xl[1], False)[None, :, None]
    kz = _wavenumbers(nz, xl[2], False)[:, None, None]
    k2 = (kx * kx + ky * ky) + kz * kz
    kmag = np.sqrt(k2)
    fac = np.ones(nh)
    fac[0] = 0.5
    fac[-1] = 0.5
    fac = np.broadcast_to(fac[None, None, :], k2.shape)

    r, _ = lcg_stream(seed, 6 * nz * ny * nh)
    r = r.reshape(nz, ny, nh, 6).astype(np.float64) - 0.5
    u = [r[..., 2 * c] + 1j * r[..., 2 * c + 1] for c in range(3)]
    del r
    safe = np.where(k2 > 0, k2, 1.0)
    div = (kx * u[0] + ky * u[1] + kz * u[2]) / safe
    u = [u[0] - div * kx, u[1] - div * ky, u[2] - div * kz]
    for c in range(3):
        u[c][0, 0, 0] = 0.0

    shell = np.floor(kmag + 0.5).astype(np.int64)
    nshell = int(shell.max()) + 1
    e_sh = np.zeros(nshell)
    np.add.at(e_sh, shell.ravel(), (fac * (np.abs(u[0]) ** 2 + np.abs(u[1]) ** 2 + np.abs(u[2]) ** 2)).ravel())
    s = np.arange(nshell, dtype=np.float64)
    target = s ** 4 * np.exp(-2.0 * (s / kpeak) ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        gain = np.where(e_sh > 0, np.sqrt(target / np.where(e_sh > 0, e_sh, 1.0)), 0.0)
    g = gain[shell]
    u = [u[c] * g for c in range(3)]

    shape = (nz, ny, nx)
    u = [sfft.rfftn(sfft.irfftn(u[c], s=shape, axes=(0, 1, 2), norm="forward"),
                    axes=(0, 1, 2), norm="forward") for c in range(3)]

    ikx, iky, ikz = kx / safe, ky / safe, kz / safe
    b = [1j * (iky * u[2] - ikz * u[1]), 1j * (ikz * u[0] - ikx * u[2]), 1j * (ikx * u[1] - iky * u[0])]
    for c in range(3):
        b[c][0, 0, 0] = 0.0
    if truncate == 1:
        kxs_max = kx[0, 0, -1] ** 2
        kys_max = ky[0, ny // 2, 0] ** 2
        kzs_max = kz[nz // 2, 0, 0] ** 2
        k1 = ((kz * kz) / kzs_max + (ky * ky) / kys_max) + (kx * kx) / kxs_max
        m = np.broadcast_to(k1 > rtrunc * rtrunc, k2.shape)
        for c in range(3):
            b[c][m] = 0.0
            b[c][0, 0, 0] = 0.0

    cu = [1j * (ky * b[2] - kz * b[1]), 1j * (kz * b[0] - kx * b[2]), 1j * (kx * b[1] - ky * b[0])]
    e = float(sum((np.where(k2 > 0, fac * np.abs(cu[c]) ** 2, 0.0)).sum() for c in range(3)))
    scale = math.sqrt(e0 / e) if e > 0 else 0.0
    return [np.ascontiguousarray(b[c] * scale) for c in range(3)]
