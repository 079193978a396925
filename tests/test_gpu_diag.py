"""Spectral diagnostics (diagnostics.f90) through the C-ABI against the oracle."""
import numpy as np
import pytest

from _helpers import configs, initial

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,phys", [((32, 32, 32), dict()), ((32, 16, 64), dict(alpnu=2.0, mu=0.1, alpmu=-1.0))])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_diagnostics_vs_oracle(lib, n, phys, precision, tol):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle, glob, helicity, spectrum, fluxes
    gp, op = configs(n, precision=precision, forcing="none", **phys)
    b = initial(n, seed=7)
    orc = Oracle(op)
    gref = glob(b, op, orc.wk)
    sp, sp2 = spectrum(b, op, orc.wk)
    n1 = orc.nlt(b, b)
    fl = fluxes(b, n1, op, orc.wk)
    h = helicity(b, op, orc.wk)
    with g.Simulation(gp) as sim:
        sim.set_state(b)
        d = sim.diagnostics(flux=True)
    np.testing.assert_allclose(d["energy"], gref["energy"], rtol=tol, atol=1e-30)
    np.testing.assert_allclose(d["enstrophy"], gref["enstrophy"], rtol=tol, atol=1e-30)
    np.testing.assert_allclose(d["spectrum"], sp, rtol=tol, atol=tol * sp.max())
    np.testing.assert_allclose(d["spectrum2d"], sp2, rtol=tol, atol=tol * max(sp2.max(), 1e-300))
    scale = np.abs(fl).max()
    np.testing.assert_allclose(d["flux"], fl, rtol=1e-3 if precision == "mixed" else 1e-9,
                               atol=(1e-4 if precision == "mixed" else 1e-10) * scale)
    assert abs(d["helicity"] - h) <= tol * 10 * (abs(h) + 1e-3 * gref["enstrophy"][:3].sum())
    assert d["nonfinite"] == 0


def test_diagnostics_bitwise_reproducible(lib):
    import gturbo3d_gb300 as g
    gp, _ = configs(64, forcing="none")
    with g.Simulation(gp) as sim:
        sim.set_state(initial(64, seed=8))
        d1 = sim.diagnostics()
        d2 = sim.diagnostics()
    for k in ("energy", "enstrophy", "spectrum", "spectrum2d", "flux"):
        assert np.array_equal(d1[k], d2[k]), k
    assert d1["helicity"] == d2["helicity"]


def test_nonfinite_state_is_reported(lib):
    """A NaN in the host input is reported as GT_ENONFINITE (failure injected
    on the host; no device fault)."""
    import gturbo3d_gb300 as g
    from gturbo3d_gb300 import _lib
    gp, _ = configs(16, forcing="none")
    b = initial(16, seed=9)
    b[1][3, 4, 5] = np.nan
    with g.Simulation(gp) as sim:
        sim.set_state(b)
        assert sim.check_finite() == _lib.GT_ENONFINITE
        sim.set_state(initial(16, seed=9))
        assert sim.check_finite() == _lib.GT_OK
