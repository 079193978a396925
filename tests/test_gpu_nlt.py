"""The fused nonlinear term nlt (nlt.f90) through the C-ABI against the oracle."""
import numpy as np
import pytest

from _helpers import configs, initial, relerr

pytestmark = pytest.mark.gpu

CASES = [
    ((16, 16, 16), dict()),
    ((32, 32, 32), dict()),
    ((32, 16, 8), dict()),
    ((8, 16, 32), dict(omega=0.0)),
    ((32, 32, 32), dict(truncate=0)),
    ((16, 32, 64), dict(omega=-3.0, truncate=0)),
    ((64, 64, 16), dict(xlz=2 * np.pi / 4)),
]


@pytest.mark.parametrize("n,phys", CASES)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-5)])
def test_nlt_vs_oracle(lib, n, phys, precision, tol):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle
    gp, op = configs(n, precision=precision, forcing="none", **phys)
    b = initial(n, seed=3)
    a = [0.8 * b[c] + 0.3 * np.roll(b[(c + 1) % 3], 1, axis=1) for c in range(3)]
    if op.truncate == 0:   # give the non-truncated case content at every mode
        rng = np.random.default_rng(4)
        a = [x + 1e-3 * (rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape)) for x in a]
        # the kx = 0 and kx = NX/2 planes of a real field are Hermitian: project them
        from oracle.gturbo_oracle import fft_dir, fft_inv
        a = [fft_dir(fft_inv(x, op), op) for x in a]
    orc = Oracle(op)
    ref = orc.nlt(a, b)
    with g.Simulation(gp) as sim:
        sim.set_state(b)
        got = sim.nlt(a)
    assert relerr(got, ref) < tol


def test_nlt_is_quadratic_plus_linear(lib):
    """With omega = 0, N(2a) = 4 N(a) (u x w is quadratic in a) — checked at
    256^3 where the oracle would be slow."""
    import gturbo3d_gb300 as g
    gp, _ = configs(256, forcing="none", omega=0.0)
    b = initial(256, seed=5)
    with g.Simulation(gp) as sim:
        n1 = sim.nlt(b)
        n2 = sim.nlt([2 * x for x in b])
    assert relerr(n2, [4 * x for x in n1]) < 1e-13
