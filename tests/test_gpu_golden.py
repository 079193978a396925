"""The library against the committed golden traces (tests/golden/*.npz,
generated by tests/golden/make_golden.py from the oracle)."""
from pathlib import Path

import numpy as np
import pytest

from _helpers import relerr

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", ["trace16_3d3c_rk2", "trace16_2d2c_as_built", "trace_32x16x8_3d3c_rk2"])
def test_trace_against_golden(lib, name):
    import gturbo3d_gb300 as g
    d = np.load(GOLD / f"{name}.npz")
    n = tuple(int(v) for v in d["shape"])
    forcing = "2d2c" if "2d2c" in name else "3d3c"
    dt2 = "as_built" if "as_built" in name else "rk2"
    phys = dict(nu=5e-3, omega=2.0) if "32x16x8" in name else {}
    p = g.make_params(*n, forcing=forcing, dt2_mode=dt2, famp=float(d["famp"]), **phys)
    b0 = list(d["b0"])
    with g.Simulation(p) as sim:
        sim.set_state(b0)
        assert relerr(sim.nlt(b0), list(d["nlt_b0"])) < 1e-12
        diag = sim.diagnostics(flux=True)
        np.testing.assert_allclose(diag["energy"], d["glob_energy"], rtol=1e-12)
        np.testing.assert_allclose(diag["enstrophy"], d["glob_enstrophy"], rtol=1e-12)
        np.testing.assert_allclose(diag["spectrum"], d["spectrum"], rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(diag["flux"], d["flux"], rtol=1e-9, atol=1e-12 * np.abs(d["flux"]).max())
        seed = int(d["seed0"])
        done = 0
        for k in (1, 2, 5):
            seed = sim.step(k - done, seed)
            done = k
            assert seed == int(d[f"seed_{k}"])
            assert relerr(sim.get_state(), list(d[f"b_{k}"])) < 1e-12
