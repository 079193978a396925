"""Host-side C-ABI checks that need no GPU: the library loads and exports
every declared symbol, the host set-up matches the oracle bit for bit, file
formats round-trip, and failures are reported as status codes."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_exports_every_declared_symbol(lib):
    hdr = (ROOT / "include" / "gturbo_gb.h").read_text()
    names = set(re.findall(r"^\s*(?:int|const char\*)\s+(gt_\w+)\s*\(", hdr, re.M))
    assert len(names) >= 30
    for n in sorted(names):
        assert hasattr(lib, n), n
    from gturbo3d_gb300._lib import SIGNATURES
    assert names == set(SIGNATURES), names ^ set(SIGNATURES)


def test_rann_matches_oracle(lib):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import rann_stream, rann
    for seed in (8299396, 0, 1, 2, 12345, 2147483646):
        v, s = g.rann(seed, 1000)
        ref, sref = rann_stream(seed, 1000)
        assert s == sref
        assert np.array_equal(v, ref)
        x = seed
        for i in range(5):
            x, r = rann(x)
            assert r == v[i]


@pytest.mark.parametrize("kind,k1f,k2f,nf_expected", [("3d3c", 1.999, 3.0, 48), ("3d3c", 2.0, 3.0, 45),
                                                       ("2d2c", 1.999, 3.0, 10)])
def test_forced_mode_counts(lib, kind, k1f, k2f, nf_expected):
    """Lattice-point counts of the forced shells in the half space (known answers
    from counting integer wavevectors with k1f < |k| <= k2f)."""
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Params, defk, iniforcing
    p = g.make_params(64, forcing=kind, k1f=k1f, k2f=k2f, famp=0.5)
    fm = g.forced_modes(p)
    assert fm.nf == nf_expected
    op = Params(nx=64, ny=64, nz=64, forcing=kind, k1f=k1f, k2f=k2f, famp=0.5)
    ofm = iniforcing(op, defk(op))
    assert np.array_equal(fm.ix, ofm.ix) and np.array_equal(fm.iy, ofm.iy) and np.array_equal(fm.iz, ofm.iz)
    assert np.array_equal(fm.ff, ofm.ff)
    assert fm.inpe == ofm.inpe and fm.inpz == ofm.inpz
    assert abs(fm.inpe - nf_expected * 0.25) < 1e-12


@pytest.mark.parametrize("kind", ["3d3c", "2d2c"])
@pytest.mark.parametrize("n", [(16, 16, 16), (32, 16, 64)])
def test_forcing_increments_bit_exact(lib, kind, n):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Params, defk, iniforcing, forcing_increments
    p = g.make_params(*n, forcing=kind, famp=0.07)
    op = Params(nx=n[0], ny=n[1], nz=n[2], forcing=kind, famp=0.07)
    wk = defk(op)
    fm = iniforcing(op, wk)
    seed = seed0 = 8299396
    for _ in range(3):
        ix, iy, iz, dF, seed = g.forcing_increments(p, seed)
        ent, seed0 = forcing_increments(op, wk, fm, seed0)
        assert seed == seed0
        assert len(ent) == len(ix)
        for e, (k, j, i, inc) in enumerate(ent):
            assert (ix[e], iy[e], iz[e]) == (i, j, k)
            for c in range(3):
                if inc[c] is None:
                    assert dF[e, 2 * c] == 0 and dF[e, 2 * c + 1] == 0
                else:
                    assert dF[e, 2 * c] == inc[c][0] and dF[e, 2 * c + 1] == inc[c][1]


def test_nforc_overflow_is_reported(lib):
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    p = g.make_params(64, k1f=0.5, k2f=20.0)
    with pytest.raises(_lib.GturboError) as ei:
        g.forced_modes(p)
    assert ei.value.code == _lib.GT_ENFORC


@pytest.mark.parametrize("bad", [dict(nx=48), dict(nx=4), dict(nz=2048), dict(dt=-1.0), dict(truncate=2),
                                 dict(forcing=7), dict(precision=3), dict(rtrunc=0.0), dict(nu=float("nan"))])
def test_invalid_params_rejected(lib, bad):
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    p = g.make_params(16)
    for k, v in bad.items():
        setattr(p, k, v)
    assert lib.gt_params_validate(C.byref(p)) == _lib.GT_EINVAL
    h = C.c_void_p()
    assert lib.gt_create(C.byref(p), C.byref(h)) == _lib.GT_EINVAL


def test_params_dat_reader(lib, tmp_path):
    """The six list-directed lines of params.dat (inieuler.f90:14-20), with
    Fortran 'd' exponents, tabs and a trailing legend."""
    import gturbo3d_gb300 as g
    f = tmp_path / "params.dat"
    f.write_text("6.2831853071795864769d0\t6.2831853071795864769d0\t3.14159265358979323846d0\n"
                 "2d-3\t1.0d0\t0.0d0\t0.0d0\n"
                 "5.0d-3\t5.0d0\n"
                 "100\t50\t10\n"
                 "0.6666666666666666667d0\t1\n"
                 "2.5d-2  1.999d0, 3.0d0\n\n"
                 "xlx   yly\nnu    alpnu\tmu\talpmu\n")
    p = g.read_params(str(f), g.make_params(64))
    assert p.xlx == 2 * np.pi and p.xlz == np.pi
    assert p.nu == 2e-3 and p.alpnu == 1.0 and p.dt == 5e-3 and p.omega == 5.0
    assert p.rtrunc == 0.6666666666666666667 and p.truncate == 1
    assert p.famp == 2.5e-2 and p.k1f == 1.999 and p.k2f == 3.0
    assert p.nx == 64


def test_params_dat_errors(lib, tmp_path):
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    with pytest.raises(_lib.GturboError) as ei:
        g.read_params(str(tmp_path / "missing.dat"))
    assert ei.value.code == _lib.GT_EIO
    f = tmp_path / "bad.dat"
    f.write_text("1 2 3\n4 5 six 7\n")
    with pytest.raises(_lib.GturboError) as ei:
        g.read_params(str(f))
    assert ei.value.code == _lib.GT_EIO
    f.write_text("1 2 3\n")
    with pytest.raises(_lib.GturboError):
        g.read_params(str(f))


def test_seed_and_field_files_round_trip(lib, tmp_path):
    import gturbo3d_gb300 as g
    g.write_seed(str(tmp_path / "seed.001"), 8299396)
    assert g.read_seed(str(tmp_path / "seed.001")) == 8299396
    u = np.random.default_rng(0).standard_normal((8, 16, 32)).astype(np.float32)
    g.write_field(str(tmp_path / "ux.001"), u)
    raw = (tmp_path / "ux.001").read_bytes()
    n = u.size * 4
    assert len(raw) == n + 8
    assert int.from_bytes(raw[:4], "little") == n and int.from_bytes(raw[-4:], "little") == n
    assert np.array_equal(np.frombuffer(raw[4:-4], np.float32).reshape(u.shape), u)
    assert np.array_equal(g.read_field(str(tmp_path / "ux.001"), 32, 16, 8), u)


def test_curframe_round_trip_and_reference_forms(lib, tmp_path):
    """curframe.dat (main.f90:37-39, 212-215): what gt_frame_write writes
    reads back exactly; list-directed forms a Fortran write or an edited file
    holds (blanks, a comma, a 'd' exponent) read too; a missing or short file
    is GT_EIO."""
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    f = tmp_path / "curframe.dat"
    g.write_frame(str(f), 7, 0.1 + 0.2)
    assert g.read_frame(str(f)) == (7, 0.1 + 0.2)
    for text, want in [("           3   1.5000000000000000     \n", (3, 1.5)),
                       ("12, 2.5d-1\n", (12, 0.25)), ("0 0.d0\n", (0, 0.0))]:
        f.write_text(text)
        assert g.read_frame(str(f)) == want
    f.write_text("4\n")
    with pytest.raises(_lib.GturboError) as ei:
        g.read_frame(str(f))
    assert ei.value.code == _lib.GT_EIO
    with pytest.raises(_lib.GturboError) as ei:
        g.read_frame(str(tmp_path / "missing.dat"))
    assert ei.value.code == _lib.GT_EIO


def test_field_file_errors(lib, tmp_path):
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    f = tmp_path / "short"
    f.write_bytes((64).to_bytes(4, "little") + b"\0" * 10)
    with pytest.raises(_lib.GturboError) as ei:
        g.read_field(str(f), 4, 4, 1)
    assert ei.value.code == _lib.GT_EIO
    with pytest.raises(_lib.GturboError):
        g.read_field(str(tmp_path / "none"), 4, 4, 1)


def test_create_without_gpu_fails_loudly(lib):
    """On a machine without a usable GPU the compute path reports GT_ECUDA
    (there is no CPU fallback)."""
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(_lib.GturboError) as ei:
        g.Simulation(nx=16)
    assert ei.value.code == _lib.GT_ECUDA


def test_memory_estimate(lib):
    import gturbo3d_gb300 as g
    p = g.make_params(512, precision="mixed")
    n = C.c_size_t()
    assert lib.gt_memory_estimate(C.byref(p), C.byref(n)) == 0
    assert 12 * 512 * 512 * 257 * 8 <= n.value < 8e9


@pytest.mark.parametrize("shape,seed", [((16, 16, 16), 8299396), ((32, 16, 8), 1), ((8, 8, 8), -5)])
def test_init_noise_matches_oracle(lib, shape, seed):
    """The fresh-start noise (trunc.f90:75-93) is bit-exact to the oracle's,
    with the seed advanced by 3 NX NY NZ draws; the library draws the stream
    in parallel chunks by LCG jump-ahead, the oracle in one pass."""
    import gturbo3d_gb300 as g
    from oracle import gturbo_oracle as O
    nx, ny, nz = shape
    p = g.make_params(nx, ny, nz, dt=5e-3)
    u, s = g.init_noise(p, seed)
    ou, os_ = O.init_noise(O.Params(nx=nx, ny=ny, nz=nz, dt=5e-3), seed)
    assert s == os_
    for c in range(3):
        assert np.array_equal(u[c], ou[c])
    # the first point's three draws, by hand from rann
    r, _ = g.rann(seed, 3)
    sdt = np.sqrt(5e-3)
    assert [u[c][0, 0, 0] for c in range(3)] == [sdt * float(np.float32(x) - np.float32(0.5)) for x in r]


def test_init_noise_large_grid_uses_jump_ahead(lib):
    """A grid large enough for the threaded path (64^3 x 3 draws) gives the
    oracle's stream too, including the chunk boundaries."""
    import gturbo3d_gb300 as g
    from oracle import gturbo_oracle as O
    p = g.make_params(128, 64, 64, dt=1e-3)
    u, s = g.init_noise(p, 12345)
    ou, os_ = O.init_noise(O.Params(nx=128, ny=64, nz=64, dt=1e-3), 12345)
    assert s == os_
    assert all(np.array_equal(u[c], ou[c]) for c in range(3))


def test_memory_budget_rejects_grid_on_host(lib):
    """A grid whose device footprint is over the budget set with
    gt_set_memory_budget gets GT_ENOMEM from gt_create, decided on the host
    before any CUDA call (so this runs without a GPU), and leaves no handle;
    the member check of gt_ensemble_create is the same one."""
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    p = g.make_params(512, precision="mixed")
    need = g.memory_estimate(p)
    assert g.memory_budget() == 0
    try:
        g.set_memory_budget(need - 1)
        assert g.memory_budget() == need - 1
        with pytest.raises(_lib.GturboError) as ei:
            g.Simulation(p)
        assert ei.value.code == _lib.GT_ENOMEM
        assert "budget" in lib.gt_last_error().decode()
        with pytest.raises(_lib.GturboError) as ei:
            g.Ensemble([g.make_params(16), p])
        assert ei.value.code == _lib.GT_ENOMEM
    finally:
        g.set_memory_budget(0)
    assert g.memory_budget() == 0


@pytest.mark.parametrize("text", ["3.0 1.5\n", "1e3 1.5\n", "99999999999 1.5\n", "-2147483649 1.5\n",
                                  "inf 1.5\n", "nan 1.5\n", "+ 1.5\n"])
def test_integer_items_are_strict(lib, tmp_path, text):
    """Integer items (frame number, seed, npas, truncate) take an optional
    sign and digits within the int32 range, as a Fortran integer read does;
    anything else is GT_EIO rather than a silent conversion."""
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    f = tmp_path / "curframe.dat"
    f.write_text(text)
    with pytest.raises(_lib.GturboError) as ei:
        g.read_frame(str(f))
    assert ei.value.code == _lib.GT_EIO
    f.write_text(text.split()[0] + "\n")
    with pytest.raises(_lib.GturboError) as ei:
        g.read_seed(str(f))
    assert ei.value.code == _lib.GT_EIO


def test_integer_item_limits(lib, tmp_path):
    import gturbo3d_gb300 as g
    f = tmp_path / "seed"
    for v in (2147483647, -2147483648, 0, 7):
        f.write_text(f"  {v}\n")
        assert g.read_seed(str(f)) == v
    f.write_text("+42\n")
    assert g.read_seed(str(f)) == 42
