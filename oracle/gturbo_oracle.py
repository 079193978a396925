"""CPU FP64 restatement of Gturbo3D's RK2 integrating-factor step (NumPy/SciPy).

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA library: the
parity tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it; nothing in the shipped ``gturbo3d_gb300`` package
does.  It follows the reference Fortran line by line (citations are
``src/<file>.f90:<line>`` within the Gturbo3D repository).

Parity status: parity unpinned against the reference itself.  The reference
needs nvfortran + OpenACC + cuFFT and no Fortran compiler exists on either
machine, so it cannot run here, and it ships no tests or golden outputs.  This
restatement is pinned instead by known answers that
follow from the reference's own formulas (LCG sequence, forced-mode counts,
exact single-mode FFTs, Beltrami/ABC invariance, the closed-form linear update
of a pure-rotation mode) in ``tests/test_oracle_known_answers.py``.  The cuFFT
boundary (``fft_dir``/``fft_inv``) is restated with ``numpy.fft`` /
``scipy.fft`` (pocketfft), which uses the same sign convention and, for real
fields, the same result up to rounding.

Array layout: every spectral field is a C-ordered ``complex128[NZ, NY, NX//2+1]``
array, byte-identical to the reference's ``complex*16 (NX/2+1, NY, NZ)``
(x fastest).  Physical fields are ``float64[NZ, NY, NX]``.  Indices here are
0-based: Fortran ``i`` is ``ix + 1``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

try:  # scipy.fft is pocketfft with a thread pool; numpy.fft is the fallback
    import scipy.fft as _sfft
except Exception:  # pragma: no cover
    _sfft = None

# Literal constants exactly as the reference spells them.
PI_REF = 3.14159265358979323846          # defk.f90:24, forcing_3d3c.f90:21
PI2_3D3C = 2.0 * 3.14159265358979323846  # forcing_3d3c.f90:21
PI2_2D2C = 2.0 * 3.14159265358979        # forcing_2d2c.f90:20 (truncated literal)
LCG_MUL = 69069                           # forcing_3d3c.f90:89
LCG_MASK = 0x7FFFFFFF                     # forcing_3d3c.f90:88
NFORC = 2048                              # modules.f90:38


@dataclass
class Params:
    """The values the reference reads from ``params.dat`` (inieuler.f90:14-20)
    plus the compile/link-time choices (grid: modules.f90:4; forcing variant:
    Makefile:20-33) and the ``dt2`` choice (rkstep.f90:30-48 reads a ``dt2``
    that nothing assigns, so the as-built value is 0)."""

    nx: int = 64
    ny: int = 64
    nz: int = 64
    xlx: float = 2.0 * PI_REF
    xly: float = 2.0 * PI_REF
    xlz: float = 2.0 * PI_REF
    nu: float = 2e-3
    alpnu: float = 1.0
    mu: float = 0.0
    alpmu: float = 0.0
    dt: float = 5e-3
    omega: float = 5.0
    rtrunc: float = 0.6666666666666666667
    truncate: int = 1
    famp: float = 0.0
    k1f: float = 1.999
    k2f: float = 3.0
    forcing: str = "3d3c"        # "3d3c" | "2d2c" | "none"
    dt2_mode: str = "rk2"        # "rk2" (dt2 = dt/2) | "as_built" (dt2 = 0)

    @property
    def nh(self) -> int:
        return self.nx // 2 + 1

    @property
    def dt2(self) -> float:
        return 0.5 * self.dt if self.dt2_mode == "rk2" else 0.0

    @property
    def sdt(self) -> float:      # inieuler.f90:67
        return math.sqrt(self.dt)


@dataclass
class Wavenumbers:
    """Tables built by ``defk`` (defk.f90:1-94)."""

    fkx: np.ndarray
    fky: np.ndarray
    fkz: np.ndarray
    fkxs: np.ndarray
    fkys: np.ndarray
    fkzs: np.ndarray
    jc: np.ndarray                # 0-based conjugate index in y
    kc: np.ndarray                # 0-based conjugate index in z
    emk: np.ndarray               # float64[NZ, NY, NH]
    fkxsmax: float
    fkysmax: float
    fkzsmax: float
    rtrunc2: float                # rtrunc squared in place (defk.f90:91)
    k2: np.ndarray = field(repr=False, default=None)   # (fkxs+fkys)+fkzs, [NZ,NY,NH]


def defk(p: Params) -> Wavenumbers:
    """Wavenumbers, conjugate maps and the integrating factor (defk.f90:13-91)."""
    nx, ny, nz, nh = p.nx, p.ny, p.nz, p.nh
    # defk.f90:13-21 (0-based: jc(0)=0, jc(j)=NY-j)
    jc = np.array([0] + [ny - j for j in range(1, ny)], dtype=np.int64)
    kc = np.array([0] + [nz - k for k in range(1, nz)], dtype=np.int64)
    # defk.f90:24-26
    dkx = 2.0 * PI_REF / p.xlx
    dky = 2.0 * PI_REF / p.xly
    dkz = 2.0 * PI_REF / p.xlz
    # defk.f90:29-43
    fkx = np.array([float(i) * dkx for i in range(nh)])
    fky = np.array([float(j) * dky if j <= ny // 2 else float(j - ny) * dky for j in range(ny)])
    fkz = np.array([float(k) * dkz if k <= nz // 2 else float(k - nz) * dkz for k in range(nz)])
    # defk.f90:46-54
    fkxs, fkys, fkzs = fkx * fkx, fky * fky, fkz * fkz
    # defk.f90:57-68: fk2 summed x, then y, then z
    k2 = (fkxs[None, None, :] + fkys[None, :, None]) + fkzs[:, None, None]
    # emk depends on fk2 alone: evaluate libm pow/exp (the host C library, as
    # the compiled reference does) once per distinct fk2.
    # "-0.5*dt*scra": the REAL*4 literal 0.5 is exact, product order ((-0.5*dt)*scra)
    uk, inv = np.unique(k2, return_inverse=True)
    ue = np.empty_like(uk)
    for n, v in enumerate(uk.tolist()):
        if v == 0.0:
            ue[n] = 1.0
        else:
            scra = p.nu * math.pow(v, p.alpnu) + p.mu * math.pow(v, p.alpmu)
            ue[n] = math.exp((-0.5 * p.dt) * scra)
    emk = ue[inv].reshape(k2.shape)
    # defk.f90:88-91
    fkxsmax = float(fkxs[nh - 1])
    fkysmax = float(fkys[ny // 2])
    fkzsmax = float(fkzs[nz // 2])
    rtrunc2 = p.rtrunc * p.rtrunc
    return Wavenumbers(fkx, fky, fkz, fkxs, fkys, fkzs, jc, kc, emk,
                       fkxsmax, fkysmax, fkzsmax, rtrunc2, k2)


# --------------------------------------------------------------------------
# Random numbers: rann (forcing_3d3c.f90:82-93)
# --------------------------------------------------------------------------

def lcg_next(irand: int) -> int:
    """irand = iand(69069*irand + 1, '7FFFFFFF'X) with 32-bit wraparound
    (forcing_3d3c.f90:88-89).  The low 31 bits of a 32-bit wrapped product are
    the product modulo 2**31, so the state evolves modulo 2**31."""
    return (LCG_MUL * irand + 1) & LCG_MASK


def rann(irand: int) -> tuple[int, np.float32]:
    """One draw: advances the state and returns REAL*4(dble(irand)/dble(mask))
    (forcing_3d3c.f90:82-93).  Returns (new_state, value)."""
    irand = lcg_next(irand)
    return irand, np.float32(float(irand) / float(LCG_MASK))


def rann_stream(seed: int, n: int) -> tuple[np.ndarray, int]:
    """``n`` consecutive ``rann`` values from state ``seed`` (vectorised with
    LCG jump-ahead: x[m*B + j] = A^m x[j] + C_m mod 2^31).  Returns (float32
    values, final state)."""
    seed = int(seed) & 0xFFFFFFFF
    if seed & 0x80000000:       # a negative 32-bit seed: 69069*seed+1 wraps the same way mod 2^31
        seed -= 1 << 32
    if n <= 0:
        return np.zeros(0, np.float32), seed
    B = min(n, 4096)
    first = np.empty(B, dtype=np.uint64)
    x = seed
    for j in range(B):
        x = lcg_next(x)
        first[j] = x
    nblk = (n + B - 1) // B
    out = np.empty(nblk * B, dtype=np.uint64)
    out[:B] = first
    # block jump: x_{j+B} = A x_j + C (mod 2^31)
    A, C = 1, 0
    for _ in range(B):
        A, C = (LCG_MUL * A) & LCG_MASK, (LCG_MUL * C + 1) & LCG_MASK
    A64, C64, M = np.uint64(A), np.uint64(C), np.uint64(LCG_MASK)
    cur = first
    for m in range(1, nblk):
        cur = (A64 * cur + C64) & M    # A < 2^31, cur < 2^31: product < 2^62
        out[m * B:(m + 1) * B] = cur
    out = out[:n]
    vals = (out.astype(np.float64) / float(LCG_MASK)).astype(np.float32)
    return vals, int(out[-1])


# --------------------------------------------------------------------------
# Forced-mode enumeration (iniforcing_3d3c.f90:16-184, iniforcing_2d2c.f90:14-73)
# --------------------------------------------------------------------------

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


def _forced_mode_ok(p, wk, ix, iy, iz, k2n_order):
    k2 = (wk.fkxs[ix] + wk.fkys[iy]) + wk.fkzs[iz]
    # iniforcing_*.f90: k2n summed x, then y, then z
    k2n = (wk.fkxs[ix] / wk.fkxsmax + wk.fkys[iy] / wk.fkysmax) + wk.fkzs[iz] / wk.fkzsmax
    ok = (k2n <= wk.rtrunc2) and (k2 <= p.k2f ** 2) and (k2 > p.k1f ** 2)
    return ok, k2


def iniforcing_3d3c(p: Params, wk: Wavenumbers) -> ForcedModes:
    """Ordered list of forced half-space modes, 3D3C (iniforcing_3d3c.f90:22-184).
    The order fixes the order of the forcing RNG draws."""
    nx2, ny2, nz2 = p.nx // 2, p.ny // 2, p.nz // 2
    order = []
    # :22-43  i=1, j=1, k=2..NZ2
    order += [(0, 0, k) for k in range(1, nz2)]
    # :45-66  i=1, j=2..NY2 (outer), k=1..NZ (inner)
    order += [(0, j, k) for j in range(1, ny2) for k in range(p.nz)]
    # :68-88  i=1, j=NY2P1, k=2..NZ2
    order += [(0, ny2, k) for k in range(1, nz2)]
    # :91-114 i=2..NX2, j=1..NY, k=1..NZ
    order += [(i, j, k) for i in range(1, nx2) for j in range(p.ny) for k in range(p.nz)]
    # :117-139 i=NX2P1, j=1, k=2..NZ2
    order += [(nx2, 0, k) for k in range(1, nz2)]
    # :141-162 i=NX2P1, j=2..NY2, k=1..NZ
    order += [(nx2, j, k) for j in range(1, ny2) for k in range(p.nz)]
    # :164-184 i=NX2P1, j=NY2P1, k=2..NZ2
    order += [(nx2, ny2, k) for k in range(1, nz2)]
    return _collect(p, wk, order, inline_inputs=True)


def iniforcing_2d2c(p: Params, wk: Wavenumbers) -> ForcedModes:
    """Ordered list of forced modes at kz=0, 2D2C (iniforcing_2d2c.f90:17-73)."""
    nx2, ny2 = p.nx // 2, p.ny // 2
    order = [(0, j, 0) for j in range(1, ny2)]                                  # :17-32
    order += [(i, j, 0) for i in range(1, nx2) for j in range(p.ny)]            # :34-50
    order += [(nx2, j, 0) for j in range(1, ny2)]                               # :52-67
    return _collect(p, wk, order, inline_inputs=False)


def _collect(p, wk, order, inline_inputs):
    ix, iy, iz, ff = [], [], [], []
    inpe = 0.0
    inpz = 0.0
    k2s = []
    for (i, j, k) in order:
        ok, k2 = _forced_mode_ok(p, wk, i, j, k, None)
        if not ok:
            continue
        if len(ix) + 1 > NFORC:
            raise ValueError("NFORC too small !")       # iniforcing_3d3c.f90:33
        kk = math.sqrt(k2)
        f = 1.0 / kk
        ix.append(i); iy.append(j); iz.append(k); ff.append(f)
        k2s.append(k2)
        if inline_inputs:                              # iniforcing_3d3c.f90:38-39
            inpz = inpz + k2 * k2 * (p.famp * f) ** 2
            inpe = inpe + k2 * (p.famp * f) ** 2
    if not inline_inputs:                              # iniforcing_2d2c.f90:69-73
        for k2, f in zip(k2s, ff):
            inpe = inpe + k2 * (p.famp * f) ** 2
            inpz = inpz + k2 * k2 * (p.famp * f) ** 2
    return ForcedModes(np.array(ix, np.int64), np.array(iy, np.int64), np.array(iz, np.int64),
                       np.array(ff, np.float64), inpe, inpz)


def iniforcing(p: Params, wk: Wavenumbers) -> ForcedModes:
    if p.forcing == "3d3c":
        return iniforcing_3d3c(p, wk)
    if p.forcing == "2d2c":
        return iniforcing_2d2c(p, wk)
    return ForcedModes(*(np.zeros(0, np.int64),) * 3, np.zeros(0), 0.0, 0.0)


# --------------------------------------------------------------------------
# Forcing (forcing_3d3c.f90:26-72, forcing_2d2c.f90:27-43)
# --------------------------------------------------------------------------

def forcing_increments(p: Params, wk: Wavenumbers, fm: ForcedModes, seed: int):
    """Draws the forcing for one step and returns (entries, new_seed).

    ``entries`` is the ordered list of scatter-adds the reference performs:
    (iz, iy, ix, [dbx, dby, dbz] complex).  Each entry is added to b in order;
    the arithmetic follows forcing_3d3c.f90:34-68 (3D3C) or
    forcing_2d2c.f90:33-41 (2D2C) operation by operation."""
    entries = []
    sf = p.sdt * p.famp
    nx2 = p.nx // 2
    for ik in range(fm.nf):
        i, j, k = int(fm.ix[ik]), int(fm.iy[ik]), int(fm.iz[ik])
        if p.forcing == "3d3c":
            seed, r = rann(seed)
            te = PI2_3D3C * float(r)
            effe = complex(sf * math.cos(te), sf * math.sin(te))
            seed, r = rann(seed)
            te = PI2_3D3C * float(r)
            cte, ste = math.cos(te), math.sin(te)
            er, ei = effe.real * fm.ff[ik], effe.imag * fm.ff[ik]    # effek = effe*ff
            if i == 0 and j == 0:                                    # :45-50
                inc = [(er * cte, ei * cte), (er * ste, ei * ste), None]
                incc = [(er * cte, -ei * cte), (er * ste, -ei * ste), None]
                entries.append((k, j, i, inc))
                entries.append((int(wk.kc[k]), int(wk.jc[j]), i, incc))
            else:                                                    # :52-68
                k2 = wk.fkxs[i] + wk.fkys[j]
                kxy = math.sqrt(k2)
                k2 = k2 + wk.fkzs[k]
                kk = math.sqrt(k2)
                c1 = wk.fkz[k] / kk
                s1 = kxy / kk
                c2 = wk.fkx[i] / kxy
                s2 = wk.fky[j] / kxy
                fx = cte * c2 * c1 - ste * s2
                fy = cte * s2 * c1 + ste * c2
                # bz - effek*cte*s1: ((effek*cte)*s1) subtracted
                inc = [(er * fx, ei * fx), (er * fy, ei * fy), (-((er * cte) * s1), -((ei * cte) * s1))]
                entries.append((k, j, i, inc))
                if i == 0 or i == nx2:
                    incc = [(er * fx, -ei * fx), (er * fy, -ei * fy),
                            (-((er * cte) * s1), -((-ei * cte) * s1))]
                    entries.append((int(wk.kc[k]), int(wk.jc[j]), i, incc))
        elif p.forcing == "2d2c":
            seed, r = rann(seed)
            te = PI2_2D2C * float(r)
            effe = complex(sf * math.cos(te), sf * math.sin(te))
            er, ei = effe.real * fm.ff[ik], effe.imag * fm.ff[ik]
            entries.append((k, j, i, [None, None, (er, ei)]))
            if i == 0 or i == nx2:
                entries.append((int(wk.kc[k]), int(wk.jc[j]), i, [None, None, (er, -ei)]))
    return entries, seed


def apply_forcing_entries(b, entries):
    """b(i,j,k) = b(i,j,k) + increment, entry by entry, in order."""
    for (k, j, i, inc) in entries:
        for c in range(3):
            if inc[c] is None:
                continue
            z = b[c][k, j, i]
            b[c][k, j, i] = complex(z.real + inc[c][0], z.imag + inc[c][1])


def forcing(p, wk, fm, b, seed):
    entries, seed = forcing_increments(p, wk, fm, seed)
    apply_forcing_entries(b, entries)
    return seed


# --------------------------------------------------------------------------
# Spectral / physical pointwise operators (produ.f90, trunc.f90, nlt.f90)
# --------------------------------------------------------------------------

def _kgrids(wk):
    return wk.fkx[None, None, :], wk.fky[None, :, None], wk.fkz[:, None, None]


def curl(a, wk):
    """u = i k x a, written out in real/imaginary parts (produ.f90:44-63)."""
    ax, ay, az = a
    kx, ky, kz = _kgrids(wk)
    xr = -ky * az.imag + kz * ay.imag
    xi = ky * az.real - kz * ay.real
    yr = -kz * ax.imag + kx * az.imag
    yi = kz * ax.real - kx * az.real
    zr = -kx * ay.imag + ky * ax.imag
    zi = kx * ay.real - ky * ax.real
    return [xr + 1j * xi, yr + 1j * yi, zr + 1j * zi]


def _cplx(re, im):
    out = np.empty(re.shape, np.complex128)
    out.real = re
    out.imag = im
    return out


def invcurl(a, wk):
    """i k x a / k^2, leaving the (0,0,0) value untouched (produ.f90:79-101)."""
    ax, ay, az = a
    k2 = wk.k2
    with np.errstate(divide="ignore", invalid="ignore"):
        kx = wk.fkx[None, None, :] / k2
        ky = wk.fky[None, :, None] / k2
        kz = wk.fkz[:, None, None] / k2
    xr = -ky * az.imag + kz * ay.imag
    xi = ky * az.real - kz * ay.real
    yr = -kz * ax.imag + kx * az.imag
    yi = kz * ax.real - kx * az.real
    zr = -kx * ay.imag + ky * ax.imag
    zi = kx * ay.real - ky * ax.real
    out = [_cplx(xr, xi), _cplx(yr, yi), _cplx(zr, zi)]
    for c in range(3):
        out[c][0, 0, 0] = a[c][0, 0, 0]
    return out


def trunc_mask(wk) -> np.ndarray:
    """True where trunc zeroes the mode: ((kz2/kzmax2 + ky2/kymax2) + kx2/kxmax2)
    > rtrunc^2 (trunc.f90:14-17), plus the (0,0,0) mode (trunc.f90:26-28)."""
    k3 = wk.fkzs[:, None, None] / wk.fkzsmax
    k2 = k3 + wk.fkys[None, :, None] / wk.fkysmax
    k1 = k2 + wk.fkxs[None, None, :] / wk.fkxsmax
    m = k1 > wk.rtrunc2
    m = np.broadcast_to(m, wk.k2.shape).copy()
    m[0, 0, 0] = True
    return m


def trunc(z, mask):
    z = z.copy()
    z[mask] = 0.0
    return z


def fft_inv(z, p: Params, workers=None):
    """Unnormalised complex-to-real 3D transform (fft_inv.f90:11-13; cuFFT Z2D
    with plan dims (NZ,NY,NX), main.f90:27)."""
    s = (p.nz, p.ny, p.nx)
    if _sfft is not None:
        return _sfft.irfftn(z, s=s, axes=(0, 1, 2), norm="forward", workers=workers)
    return np.fft.irfftn(z, s=s, axes=(0, 1, 2), norm="forward")


def fft_dir(x, p: Params, workers=None):
    """Real-to-complex 3D transform scaled by 1/(NX*NY*NZ) (fft_dir.f90:11-25).
    The reference divides by NY, NX, NZ in turn; for powers of two each
    division is exact, so this equals one multiplication by 1/(NX*NY*NZ)."""
    if _sfft is not None:
        return _sfft.rfftn(x, axes=(0, 1, 2), norm="forward", workers=workers)
    return np.fft.rfftn(x, axes=(0, 1, 2), norm="forward")


def cross(u, w):
    """(a2 b3 - a3 b2, a3 b1 - a1 b3, a1 b2 - a2 b1) (produ.f90:9-28).  The
    padding columns it zeroes do not exist in the un-padded real arrays here."""
    return [u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]]


def nlt(a, bcor, p: Params, wk: Wavenumbers, mask=None, workers=None, return_physical=False):
    """Nonlinear term N = P_trunc invcurl[FFT(u x w) + i omega kz bcor] with
    u = curl a, w = k^2 a (nlt.f90:16-89).  ``bcor`` is the state at time t in
    both RK stages (main.f90:131,144 pass ``bx,by,bz`` as the Coriolis source)."""
    v = curl(a, wk)                                   # nlt.f90:16-23
    w = [wk.k2 * a[c] for c in range(3)]              # nlt.f90:26-40 (real k2 * complex)
    ur = [fft_inv(v[c], p, workers) for c in range(3)]  # nlt.f90:44-49
    wr = [fft_inv(w[c], p, workers) for c in range(3)]
    cr = cross(ur, wr)                                # nlt.f90:55
    vh = [fft_dir(cr[c], p, workers) for c in range(3)]  # nlt.f90:59-61
    kz = wk.fkz[:, None, None]
    okz = p.omega * kz
    out = []
    for c in range(3):                                # nlt.f90:67-81
        re = vh[c].real - okz * bcor[c].imag
        im = vh[c].imag + okz * bcor[c].real
        out.append(_cplx(re, im))
    out = invcurl(out, wk)                            # nlt.f90:83
    if p.truncate == 1:                               # nlt.f90:85-89
        if mask is None:
            mask = trunc_mask(wk)
        out = [trunc(out[c], mask) for c in range(3)]
    if return_physical:
        return out, (ur, wr, cr)
    return out


def step1(a, c, p: Params, wk: Wavenumbers, zero_origin: bool = True):
    """c = emk (a + dt2 c); c(1,1,1) = 0 (rkstep.f90:30-48, split = 0).
    ``zero_origin`` = False for a z-slab that does not hold the (0,0,0) mode."""
    dt2 = p.dt2
    out = []
    for ci in range(3):
        re = wk.emk * (a[ci].real + dt2 * c[ci].real)
        im = wk.emk * (a[ci].imag + dt2 * c[ci].imag)
        z = _cplx(re, im)
        if zero_origin:
            z[0, 0, 0] = 0.0
        out.append(z)
    return out


def step2(a, c, p: Params, wk: Wavenumbers, zero_origin: bool = True):
    """a = emk (emk a + dt c); a(1,1,1) = 0 (rkstep.f90:86-104, split = 0)."""
    out = []
    for ci in range(3):
        re = wk.emk * (wk.emk * a[ci].real + p.dt * c[ci].real)
        im = wk.emk * (wk.emk * a[ci].imag + p.dt * c[ci].imag)
        z = _cplx(re, im)
        if zero_origin:
            z[0, 0, 0] = 0.0
        out.append(z)
    return out


def _slabs(nz, nthreads):
    n = max(1, min(nthreads, nz))
    edges = [nz * i // n for i in range(n + 1)]
    return [slice(edges[i], edges[i + 1]) for i in range(n)]


class _SlabWk:
    """The wavenumber tables restricted to a z-slab (for slab-parallel work)."""

    def __init__(self, wk, sl):
        self.fkx, self.fky, self.fkz = wk.fkx, wk.fky, wk.fkz[sl]
        self.k2 = wk.k2[sl]


def nlt_threaded(a, bcor, p: Params, wk: Wavenumbers, mask, nthreads: int):
    """nlt with its pointwise stages run in parallel over z-slabs (NumPy
    releases the GIL) and the FFTs on nthreads scipy workers.  Every value is
    computed by the same expression as in ``nlt``, so the result is identical."""
    from concurrent.futures import ThreadPoolExecutor
    sls = _slabs(p.nz, nthreads)
    v = [np.empty_like(a[0]) for _ in range(3)]
    w = [np.empty_like(a[0]) for _ in range(3)]

    def pre(sl):
        sw = _SlabWk(wk, sl)
        cs = curl([a[c][sl] for c in range(3)], sw)
        for c in range(3):
            v[c][sl] = cs[c]
            w[c][sl] = sw.k2 * a[c][sl]

    with ThreadPoolExecutor(len(sls)) as ex:
        list(ex.map(pre, sls))
        ur = [fft_inv(v[c], p, nthreads) for c in range(3)]
        wr = [fft_inv(w[c], p, nthreads) for c in range(3)]
        cr = [np.empty_like(ur[0]) for _ in range(3)]

        def mid(sl):
            cc = cross([x[sl] for x in ur], [x[sl] for x in wr])
            for c in range(3):
                cr[c][sl] = cc[c]

        list(ex.map(mid, sls))
        del ur, wr
        vh = [fft_dir(cr[c], p, nthreads) for c in range(3)]
        out = [np.empty_like(a[0]) for _ in range(3)]

        def post(sl):
            sw = _SlabWk(wk, sl)
            okz = p.omega * sw.fkz[:, None, None]
            t = []
            for c in range(3):
                re = vh[c][sl].real - okz * bcor[c][sl].imag
                im = vh[c][sl].imag + okz * bcor[c][sl].real
                t.append(_cplx(re, im))
            r = invcurl_slab(t, sw, sl.start == 0)
            for c in range(3):
                if p.truncate == 1:
                    r[c][mask[sl]] = 0.0
                out[c][sl] = r[c]

        list(ex.map(post, sls))
    return out


def invcurl_slab(a, sw, has_origin):
    """invcurl on a z-slab (the origin mode is left as is, as in produ.f90:83)."""
    ax, ay, az = a
    k2 = sw.k2
    with np.errstate(divide="ignore", invalid="ignore"):
        kx = sw.fkx[None, None, :] / k2
        ky = sw.fky[None, :, None] / k2
        kz = sw.fkz[:, None, None] / k2
    xr = -ky * az.imag + kz * ay.imag
    xi = ky * az.real - kz * ay.real
    yr = -kz * ax.imag + kx * az.imag
    yi = kz * ax.real - kx * az.real
    zr = -kx * ay.imag + ky * ax.imag
    zi = kx * ay.real - ky * ax.real
    out = [_cplx(xr, xi), _cplx(yr, yi), _cplx(zr, zi)]
    if has_origin:
        for c in range(3):
            out[c][0, 0, 0] = a[c][0, 0, 0]
    return out


class Oracle:
    """One simulation in the reference's order of operations (main.f90:121-150).
    ``threads`` > 1 runs the pointwise stages slab-parallel (same results)."""

    def __init__(self, p: Params, workers=None, threads: int = 1):
        self.p = p
        self.wk = defk(p)
        self.fm = iniforcing(p, self.wk)
        self.mask = trunc_mask(self.wk) if p.truncate == 1 else None
        self.workers = workers
        self.threads = threads

    def nlt(self, a, bcor):
        if self.threads > 1:
            return nlt_threaded(a, bcor, self.p, self.wk, self.mask, self.threads)
        return nlt(a, bcor, self.p, self.wk, self.mask, self.workers)

    def _stage(self, fn, a, c):
        if self.threads <= 1:
            return fn(a, c, self.p, self.wk)
        from concurrent.futures import ThreadPoolExecutor
        out = [np.empty_like(a[0]) for _ in range(3)]
        sls = _slabs(self.p.nz, self.threads)

        class _W:
            pass

        def run(sl):
            w = _W()
            w.emk = self.wk.emk[sl]
            r = fn([x[sl] for x in a], [x[sl] for x in c], self.p, w, zero_origin=(sl.start == 0))
            for ci in range(3):
                out[ci][sl] = r[ci]

        with ThreadPoolExecutor(len(sls)) as ex:
            list(ex.map(run, sls))
        return out

    def rk2_step(self, b, seed):
        """One RK2 step; returns (b_new, seed_new, n1).  ``n1`` is N(b) from the
        first nlt, which ``fluxes`` uses (main.f90:131-137)."""
        n1 = self.nlt(b, b)                       # main.f90:124-131
        c = self._stage(step1, b, n1)             # main.f90:141
        n2 = self.nlt(c, b)                       # main.f90:144
        bn = self._stage(step2, b, n2)            # main.f90:146
        if self.p.forcing in ("3d3c", "2d2c") and self.fm.nf > 0:
            seed = forcing(self.p, self.wk, self.fm, bn, seed)   # main.f90:149
        return bn, seed, n1

    def run(self, b, seed, nsteps):
        for _ in range(nsteps):
            b, seed, _ = self.rk2_step(b, seed)
        return b, seed


# --------------------------------------------------------------------------
# Diagnostics (diagnostics.f90)
# --------------------------------------------------------------------------

def _fac(p, dtype=np.float64, edge=0.5, interior=1.0):
    f = np.full(p.nh, interior, dtype)
    f[0] = edge
    f[p.nh - 1] = edge
    return f[None, None, :]


def _abs2(z):
    # cdabs(z)**2 (diagnostics.f90:225,333)
    return np.abs(z) ** 2


def glob(b, p: Params, wk: Wavenumbers):
    """Energy and enstrophy budgets (diagnostics.f90:114-199).

    Returns a dict with arrays of 9 values each: ``energy`` = [E_x, E_y, E_z,
    eps_nu_{x,y,z}, eps_mu_{x,y,z}] from u = curl b and ``enstrophy`` = the same
    from w = curl u; the k = 0 mode is excluded; fac = 0.5 on the first and last
    x-planes."""
    fac = _fac(p)
    k2 = wk.k2
    nzm = k2 > 0.0
    out = {}
    a = curl(b, wk)
    for name in ("energy", "enstrophy"):
        t = np.zeros(9)
        for c in range(3):
            s = fac * _abs2(a[c])
            s = np.where(nzm, s, 0.0)
            t[c] = s.sum()
            with np.errstate(divide="ignore", invalid="ignore"):
                t[3 + c] = np.where(nzm, 2.0 * p.nu * s * np.power(k2, p.alpnu), 0.0).sum()
                t[6 + c] = np.where(nzm, 2.0 * p.mu * s * np.power(k2, p.alpmu), 0.0).sum()
        out[name] = t
        a = curl(a, wk)
    return out


def helicity(b, p: Params, wk: Wavenumbers) -> float:
    """Kinetic helicity H = sum_k fac Re(u . conj(w)), u = curl b, w = curl u,
    k = 0 excluded, same half-spectrum weights as ``glob``.  The reference has
    no helicity diagnostic; this is the definition the library implements."""
    fac = _fac(p)
    u = curl(b, wk)
    w = curl(u, wk)
    s = sum((u[c] * np.conj(w[c])).real for c in range(3))
    s = np.where(wk.k2 > 0.0, fac * s, 0.0)
    return float(s.sum())


def spectrum(b, p: Params, wk: Wavenumbers):
    """E(k) and E_2D(k) (diagnostics.f90:22-53).  Returns two arrays of NBIN =
    NX/2 values; element s is the reference's bin ib = s+1, i.e. shell
    s <= |k| < s+1.  Shells with ib >= NBIN are dropped, as in the reference."""
    nbin = p.nx // 2
    fac = np.broadcast_to(_fac(p), wk.k2.shape)
    kk = np.sqrt(wk.k2)
    ib = kk.astype(np.int64) + 1
    scra = _abs2(b[0]) + _abs2(b[1]) + _abs2(b[2])
    val = kk * kk * fac * scra
    sel = (ib > 0) & (ib < nbin)
    sp = np.zeros(nbin)
    np.add.at(sp, ib[sel] - 1, val[sel])
    kk2 = kk[0]
    ib2 = ib[0]
    val2 = kk2 * kk2 * fac[0] * _abs2(b[2][0])
    sel2 = (ib2 > 0) & (ib2 < nbin)
    sp2d = np.zeros(nbin)
    np.add.at(sp2d, ib2[sel2] - 1, val2[sel2])
    return sp, sp2d


def fluxes(b, n1, p: Params, wk: Wavenumbers):
    """Energy flux Pi(k) (diagnostics.f90:77-100).  ``n1`` is N(b) from the first
    nlt of the step.  Element s is the reference's ib = s+1: the cumulative sum
    of shells int(|k|) >= s+1.  The reference also adds the int(|k|) = 0 shell
    at sp(0), one slot before its array (an out-of-bounds write); that shell
    holds only k = 0, whose term is k^2 * ... = 0, and it is dropped here."""
    nbin = p.nx // 2
    fac = np.full(p.nh, 2.0)
    fac[0] = 1.0
    fac[p.nh - 1] = 1.0
    fac = np.broadcast_to(fac[None, None, :], wk.k2.shape)
    kk = np.sqrt(wk.k2)
    ib = kk.astype(np.int64)
    scra = (b[0] * np.conj(n1[0]) + b[1] * np.conj(n1[1]) + b[2] * np.conj(n1[2])).real
    val = fac * kk * kk * scra
    sel = (ib >= 1) & (ib < nbin)
    sp = np.zeros(nbin + 1)          # 1-based slots 1..NBIN
    np.add.at(sp, ib[sel], val[sel])
    spf = np.array([sp[i:nbin + 1].sum() for i in range(1, nbin + 1)])
    return spf


def energy(b, p, wk) -> float:
    """Total kinetic energy E = sum of glob's three energy components."""
    return float(glob(b, p, wk)["energy"][:3].sum())


# --------------------------------------------------------------------------
# Initial-state path (main.f90:91-106, trunc.f90:47-63)
# --------------------------------------------------------------------------

def incompr(a, wk):
    """Remove the k-parallel part (trunc.f90:47-63), skipping k = 0.  Returns
    (a_new, cc) where cc = sum |k.a|^2 is the reference's 'Initial
    compressibility' (computed here as a proper reduction)."""
    ax, ay, az = a
    kx, ky, kz = _kgrids(wk)
    scra = kx * ax + ky * ay + kz * az
    k2 = wk.k2
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(k2 > 0, scra / np.where(k2 > 0, k2, 1.0), 0.0)
    cc = float(np.where(k2 > 0, np.abs(scra) ** 2, 0.0).sum())
    out = [ax - r * kx, ay - r * ky, az - r * kz]
    for c in range(3):
        out[c][0, 0, 0] = a[c][0, 0, 0]
    return out, cc


def init_noise(p: Params, seed: int):
    """The fresh-start noise (inieuler.f90:76-82, trunc.f90:75-93): the arrays
    start at zero and, for k, j, i (x fastest), b{x,y,z}(i,j,k) +=
    sdt*(rann(seed)-0.5) with the three components drawn in turn; rann - 0.5
    is REAL*4 arithmetic, promoted by the REAL*8 sdt = sqrt(dt)
    (inieuler.f90:67).  Returns ([ux, uy, uz] as float64[NZ, NY, NX], seed)."""
    n = p.nx * p.ny * p.nz
    r, seed = rann_stream(seed, 3 * n)
    d = (r - np.float32(0.5)).astype(np.float32).reshape(n, 3)
    sdt = math.sqrt(p.dt)
    return [sdt * d[:, c].astype(np.float64).reshape(p.nz, p.ny, p.nx) for c in range(3)], seed


def velocity_to_potential(ur, p, wk, mask=None):
    """main.f90:91-106: fft_dir x3, incompr, invcurl, trunc x3."""
    a = [fft_dir(ur[c], p) for c in range(3)]
    a, cc = incompr(a, wk)
    a = invcurl(a, wk)
    if p.truncate == 1:
        if mask is None:
            mask = trunc_mask(wk)
        a = [trunc(a[c], mask) for c in range(3)]
    return a, cc


def potential_to_velocity(b, p, wk):
    """main.f90:188-201: curl, then fft_inv x3 (the output path)."""
    u = curl(b, wk)
    return [fft_inv(u[c], p) for c in range(3)]
