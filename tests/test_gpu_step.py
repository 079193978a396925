"""The RK2 step (main.f90:121-150) through the C-ABI against the oracle."""
import numpy as np
import pytest

from _helpers import configs, initial, relerr

pytestmark = pytest.mark.gpu

CASES = [
    ((16, 16, 16), "3d3c", "rk2", dict()),
    ((16, 16, 16), "3d3c", "as_built", dict()),
    ((32, 32, 32), "2d2c", "rk2", dict()),
    ((32, 16, 8), "3d3c", "rk2", dict(nu=5e-3)),
    ((16, 16, 32), "none", "rk2", dict(truncate=0)),
    ((32, 32, 32), "3d3c", "rk2", dict(alpnu=2.0, nu=1e-5, mu=0.05, alpmu=-1.0)),
    ((32, 32, 16), "3d3c", "rk2", dict(xlz=2 * np.pi / 3)),
]


def _run(n, forcing, dt2, phys, precision, nsteps, seed=8299396):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle
    gp, op = configs(n, precision=precision, forcing=forcing, dt2_mode=dt2, **phys)
    if forcing != "none":
        famp = g.forcing_amplitude(0.1, gp)
        gp.famp = famp
        op.famp = famp
    b0 = initial(n, seed=1)
    orc = Oracle(op)
    bref, sref = orc.run(b0, seed, nsteps)
    with g.Simulation(gp) as sim:
        sim.set_state(b0)
        s = sim.step(nsteps, seed)
        got = sim.get_state()
    return got, bref, s, sref


@pytest.mark.parametrize("n,forcing,dt2,phys", CASES)
def test_one_step_fp64(lib, n, forcing, dt2, phys):
    got, ref, s, sref = _run(n, forcing, dt2, phys, "fp64", 1)
    assert s == sref
    assert relerr(got, ref) < 1e-12


@pytest.mark.parametrize("n,forcing,dt2,phys", CASES[:4])
def test_ten_steps_fp64(lib, n, forcing, dt2, phys):
    got, ref, s, sref = _run(n, forcing, dt2, phys, "fp64", 10)
    assert s == sref
    assert relerr(got, ref) < 1e-11


@pytest.mark.parametrize("n,forcing,dt2,phys", CASES[:4])
def test_ten_steps_mixed(lib, n, forcing, dt2, phys):
    got, ref, s, sref = _run(n, forcing, dt2, phys, "mixed", 10)
    assert s == sref
    assert relerr(got, ref) < 1e-5


@pytest.mark.slow
def test_config1_64cubed_100_steps(lib):
    """The CPU-runnable configuration: 64^3, nu=2e-3, Omega=5, dt=5e-3, 3D3C
    forcing at injection 0.1, 100 RK2 steps: FP64 state against the oracle
    (1e-9) and the mixed form's relative kinetic-energy error (1e-5)."""
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle, energy
    gp, op = configs(64, forcing="3d3c", nu=2e-3, omega=5.0, dt=5e-3)
    famp = g.forcing_amplitude(0.1, gp)
    gp.famp = op.famp = famp
    b0 = initial(64, seed=0)
    orc = Oracle(op)
    bref, sref = orc.run(b0, 0, 100)
    e_ref = energy(bref, op, orc.wk)
    with g.Simulation(gp) as sim:
        sim.set_state(b0)
        s = sim.step(100, 0)
        got = sim.get_state()
        e64 = sim.energy()
    assert s == sref
    assert relerr(got, bref) < 1e-9
    assert abs(e64 - e_ref) / e_ref < 1e-11
    gp.precision = 1
    with g.Simulation(gp) as sim:
        sim.set_state(b0)
        sim.step(100, 0)
        e32 = sim.energy()
    assert abs(e32 - e_ref) / e_ref < 1e-5


def test_host_driven_forcing_matches_seeded(lib):
    """gt_rk2_step_coeffs fed with gt_forcing_increments reproduces gt_rk2_step
    bit for bit (same device arithmetic, same increments)."""
    import gturbo3d_gb300 as g
    gp, _ = configs(32, forcing="3d3c")
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(32, seed=2)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        b.set_state(b0)
        seed = 12345
        s1 = a.step(3, seed)
        for _ in range(3):
            ix, iy, iz, dF, seed = g.forcing_increments(gp, seed)
            b.step_coeffs(ix, iy, iz, dF)
        assert s1 == seed
        xa, xb = a.get_state(), b.get_state()
    for c in range(3):
        assert np.array_equal(xa[c], xb[c])


def test_forcing_scatter_is_exact(lib):
    """With nu = 0, omega = 0 and a zero state the step leaves b = 0 and the
    forcing adds exactly the reference's increments (bitwise)."""
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle, forcing
    gp, op = configs(16, forcing="3d3c", nu=0.0, omega=0.0)
    gp.famp = op.famp = 0.3
    zero = [np.zeros((16, 16, 9), np.complex128) for _ in range(3)]
    orc = Oracle(op)
    ref = [z.copy() for z in zero]
    sref = forcing(op, orc.wk, orc.fm, ref, 77)
    with g.Simulation(gp) as sim:
        sim.set_state(zero)
        s = sim.step(1, 77)
        got = sim.get_state()
    assert s == sref
    for c in range(3):
        assert np.array_equal(got[c], ref[c])
