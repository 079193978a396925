"""The initial-state path (main.f90:91-106) and the output path
(main.f90:188-201) against the oracle."""
import numpy as np
import pytest

from _helpers import configs, initial, relerr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-6)])
def test_velocity_output_path(lib, precision, tol):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle, potential_to_velocity
    gp, op = configs((32, 16, 32), precision=precision, forcing="none")
    b = initial((32, 16, 32), seed=4)
    ref = potential_to_velocity(b, op, Oracle(op).wk)
    with g.Simulation(gp) as sim:
        sim.set_state(b)
        u = sim.velocity()
    assert relerr(u, ref) < tol


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-6)])
def test_initial_state_path(lib, precision, tol):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle, velocity_to_potential
    gp, op = configs(32, precision=precision, forcing="none")
    rng = np.random.default_rng(11)
    u = [rng.standard_normal((32, 32, 32)) for _ in range(3)]   # compressible noise
    ref, cc_ref = velocity_to_potential(u, op, Oracle(op).wk)
    with g.Simulation(gp) as sim:
        cc = sim.set_state_physical(u)
        got = sim.get_state()
    assert relerr(got, ref) < tol
    assert abs(cc - cc_ref) / cc_ref < max(tol, 1e-12) * 10


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 1e-6)])
def test_fresh_start_from_reference_noise(lib, precision, tol):
    """The reference's fresh start (inieuler.f90:76-82): the host noise of
    gt_init_noise through the device initial-state path equals the oracle's
    init_noise through its velocity_to_potential."""
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle, init_noise, velocity_to_potential
    gp, op = configs(32, precision=precision, forcing="none")
    u, seed = g.init_noise(gp, 8299396)
    ou, oseed = init_noise(op, 8299396)
    assert seed == oseed and all(np.array_equal(u[c], ou[c]) for c in range(3))
    ref, cc_ref = velocity_to_potential(ou, op, Oracle(op).wk)
    with g.Simulation(gp) as sim:
        cc = sim.set_state_physical(u)
        got = sim.get_state()
    assert relerr(got, ref) < tol
    assert abs(cc - cc_ref) / cc_ref < max(tol, 1e-12) * 10


@pytest.mark.gpu
def test_bounded_wait_times_out_and_handle_survives(lib):
    """A device wait that nothing completes gives up, reports GT_ETIMEOUT
    through the error flag, and the handle keeps stepping correctly."""
    import gturbo3d_gb300 as g
    gp, _ = configs(16, forcing="none")
    b0 = initial(16, seed=2)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        b.set_state(b0)
        assert a.selftest_wait_timeout() == -7
        assert a.selftest_wait_timeout() == -7        # the flag was cleared and set again
        a.step(2, 0)
        b.step(2, 0)
        assert relerr(a.get_state(), b.get_state()) == 0.0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_pattern_probe_leaves_the_trajectory_unchanged(lib, precision):
    """gt_probe_patterns times copy kernels in the handle's work and stage
    buffers only: a run interrupted by the probe between two steps is bitwise
    the run without it, and every pass gets a positive time."""
    import gturbo3d_gb300 as g
    n = (64, 32, 32)
    gp, _ = configs(n, precision=precision, forcing="3d3c", dt2_mode="rk2")
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=9)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        sa = a.step(2, 4242)
        b.set_state(b0)
        sb = b.step(1, 4242)
        ms = b.probe_patterns()
        sb = b.step(1, sb)
        assert sa == sb
        assert set(ms) == set(g.Simulation.PATTERN_PASSES)
        assert all(v > 0 for v in ms.values())
        for x, y in zip(a.get_state(), b.get_state()):
            assert np.array_equal(x, y)
