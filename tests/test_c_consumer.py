"""The C-ABI as a compiled consumer sees it: tests/c_consumer.c is built with
gcc -std=c11 -Wall -Werror -pedantic against include/gturbo_gb.h alone and
linked to the library; the public structs' layout must equal the Python
mirror's (the layout a Fortran bind(C) type reproduces), and the host-only
entry points must give the oracle's values.  The header must also compile as
C++ (its extern "C" guard)."""
import ctypes as C
import json
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")


@pytest.fixture(scope="module")
def consumer(lib, tmp_path_factory):
    from gturbo3d_gb300 import _lib
    d = tmp_path_factory.mktemp("cabi")
    exe = d / "c_consumer"
    libdir = _lib.LIB_PATH.parent
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "c_consumer.c"), "-o", str(exe), f"-L{libdir}", "-lgturbo_gb",
                    f"-Wl,-rpath,{libdir}"], check=True, capture_output=True, text=True)
    pdat = d / "params.dat"
    pdat.write_text("6.2831853071795864769d0 6.2831853071795864769d0 6.2831853071795864769d0\n"
                    "2d-3 1.0d0 0.0d0 0.0d0\n5.0d-3 5.0d0\n100 50 10\n0.6666666666666666667d0 1\n"
                    "0.05d0 1.999d0 3.0d0\n")
    out = subprocess.run([str(exe), str(pdat)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def test_header_compiles_as_cxx(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    src = tmp_path / "h.cpp"
    src.write_text('#include "gturbo_gb.h"\nint main() { gt_params p; return gt_params_default(&p); }\n')
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"),
                    str(src)], check=True)


@pytest.mark.parametrize("name,cls", [("gt_params", "GtParams"), ("gt_diag", "GtDiag")])
def test_struct_layout_matches_mirror(consumer, name, cls):
    from gturbo3d_gb300 import _lib
    mirror = getattr(_lib, cls)
    got = consumer[name]
    assert got["size"] == C.sizeof(mirror)
    for fname, _ in mirror._fields_:
        off, size = got[fname]
        f = getattr(mirror, fname)
        assert (off, size) == (f.offset, f.size), fname


def test_host_entry_points_from_c(consumer):
    import gturbo3d_gb300 as g
    from oracle import gturbo_oracle as O

    c = consumer
    assert c["default_rc"] == 0 and c["read_rc"] == 0 and c["validate_rc"] == 0
    assert (c["read_nu"], c["read_dt"], c["read_omega"]) == (2e-3, 5e-3, 5.0)
    assert c["estimate_rc"] == 0 and c["estimate_bytes"] > 0
    # rann: the reference LCG from seed.0 = 8299396 (forcing_3d3c.f90:82-93)
    vals, state = O.rann_stream(8299396, 5)
    assert c["rann_rc"] == 0 and c["rann_state"] == state
    assert np.array_equal(np.float32(c["rann"]), np.asarray(vals, np.float32))
    # forced modes and one step's increments: the same as through the Python mirror
    p = g.make_params(32, forcing="3d3c", nu=2e-3, omega=5.0, dt=5e-3, famp=0.05)
    fm = g.forced_modes(p)
    assert c["modes_rc"] == 0 and c["nf"] == fm.nf == 48
    assert c["first_mode"] == [int(fm.iz[0]), int(fm.iy[0]), int(fm.ix[0])]
    ix, iy, iz, dF, s = g.forcing_increments(p, 8299396)
    assert c["incr_rc"] == 0 and c["n"] == len(ix) and c["seed_after"] == s
    assert c["dF0"] == [dF[0, 0], dF[0, 1]]
    assert c["dF_sum"] == pytest.approx(float(dF.sum()), rel=1e-14, abs=1e-300)
    assert c["bad_grid_rc"] == -1 and c["strerror_einval"]
