"""Truncation-aware pruning: the pruned step equals the full step up to
rounding, and it is used exactly when the state is zero outside K."""
import numpy as np
import pytest

from _helpers import configs, initial, relerr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [(32, 32, 32), (64, 32, 16), (16, 64, 32)])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-14), ("mixed", 2e-6)])
def test_pruned_equals_full(lib, n, precision, tol):
    import gturbo3d_gb300 as g
    gp, _ = configs(n, precision=precision, forcing="3d3c")
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=6)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        b.set_state(b0)
        b.set_pruning(False)
        assert a.pruning_active and not b.pruning_active
        sa = a.step(5, 99)
        sb = b.step(5, 99)
        assert sa == sb
        assert relerr(a.get_state(), b.get_state()) < tol
        # the pruned state stays exactly zero outside K
        assert a.pruning_active


def test_pruning_follows_the_state(lib):
    import gturbo3d_gb300 as g
    gp, _ = configs(32, forcing="3d3c")
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(32, seed=6)
    with g.Simulation(gp) as sim:
        assert sim.pruning_active                      # zero state
        sim.set_state(b0)
        assert sim.pruning_active
        bad = [x.copy() for x in b0]
        bad[0][0, 0, 16] = 1e-3                        # kx = NX/2: outside K
        sim.set_state(bad)
        assert not sim.pruning_active
        sim.step(1, 5)
        assert not sim.pruning_active
        sim.set_state(b0)
        assert sim.pruning_active
    gp0, _ = configs(32, forcing="3d3c", truncate=0)
    with g.Simulation(gp0) as sim:
        sim.set_state(b0)
        assert not sim.pruning_active                  # no truncation: nothing to prune


@pytest.mark.gpu
@pytest.mark.parametrize("n,precision,tol", [(32, "fp64", 1e-13), (64, "mixed", 1e-5), (128, "mixed", 1e-5),
                                             ((8, 16, 16), "fp64", 1e-13), ((16, 32, 8), "mixed", 1e-5),
                                             ((1024, 8, 8), "mixed", 1e-5), ((1024, 8, 8), "fp64", 1e-13)])
@pytest.mark.parametrize("truncate", [1, 0])
@pytest.mark.parametrize("fused", [1, 2, 3])
def test_fused_x_pass_equals_three_group_pass(lib, n, precision, tol, truncate, fused):
    """The register-resident x pass (one thread group per row pair; 2: its
    three lines per row transformed together; 3: the same with row 0's
    products parked in shared memory) and the three-group x pass compute the
    same u x w and give the same step."""
    import gturbo3d_gb300 as g
    gp, _ = configs(n, precision=precision, forcing="3d3c", truncate=truncate)
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=9)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        b.set_state(b0)
        a.set_tuning("x_fused", fused)
        b.set_tuning("x_fused", 0)
        a.step(3, 5)
        b.step(3, 5)
        assert relerr(a.get_state(), b.get_state()) < tol




@pytest.mark.gpu
@pytest.mark.parametrize("n", [64, (16, 64, 32), (64, 1024, 8), (64, 8, 16), (8, 16, 16), (128, 32, 64)])
@pytest.mark.parametrize("truncate", [1, 0])
def test_paired_y_pass_equals_plain(lib, n, truncate):
    """FP32 y passes with two adjacent columns per thread give the result of
    the one-column-per-thread y passes (same arithmetic, bit for bit up to
    the compiler's FMA contraction)."""
    import gturbo3d_gb300 as g
    gp, _ = configs(n, precision="mixed", forcing="3d3c", truncate=truncate)
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=11)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        b.set_state(b0)
        a.set_tuning("y_pairs", 1)
        b.set_tuning("y_pairs", 0)
        a.step(3, 5)
        b.step(3, 5)
        assert relerr(a.get_state(), b.get_state()) < 1e-6



@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pruned_energy_reduction_is_exact(lib, precision):
    """The energy reduction that visits only the kept modes (state zero
    outside them) gives the full reduction bit for bit."""
    import gturbo3d_gb300 as g
    gp, _ = configs((32, 64, 16), precision=precision, forcing="3d3c")
    gp.famp = g.forcing_amplitude(0.1, gp)
    with g.Simulation(gp) as sim:
        sim.set_state(initial((32, 64, 16), seed=13))
        sim.step(2, 5)
        assert sim.pruning_active
        e_pruned = sim.energy()
        sim.set_pruning(False)
        assert not sim.pruning_active
        assert sim.energy() == e_pruned


@pytest.mark.gpu
@pytest.mark.parametrize("n,precision,tol", [(32, "fp64", 1e-13), (64, "mixed", 1e-5), ((16, 64, 32), "fp64", 1e-13),
                                             ((64, 32, 16), "mixed", 1e-5), ((8, 16, 1024), "fp64", 1e-13)])
@pytest.mark.parametrize("truncate,dt2", [(1, "rk2"), (0, "rk2"), (1, "as_built")])
def test_fused_stage_boundary_equals_separate_passes(lib, n, precision, tol, truncate, dt2):
    """The RK2 step with the first term's z forward pass and the second
    term's z inverse pass fused (c kept on chip) equals the step with c
    written to and read back from HBM."""
    import gturbo3d_gb300 as g
    gp, _ = configs(n, precision=precision, forcing="3d3c", truncate=truncate, dt2_mode=dt2)
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=14)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        b.set_state(b0)
        a.set_tuning("fuse_stage", 1)
        b.set_tuning("fuse_stage", 0)
        a.step(3, 5)
        b.step(3, 5)
        assert relerr(a.get_state(), b.get_state()) < tol


@pytest.mark.gpu
@pytest.mark.parametrize("n,precision,tol", [(32, "fp64", 1e-14), (64, "mixed", 1e-6), ((16, 64, 32), "mixed", 1e-6),
                                             ((64, 16, 1024), "fp64", 1e-14), ((8, 8, 16), "mixed", 1e-6)])
@pytest.mark.parametrize("truncate", [1, 0])
@pytest.mark.parametrize("split", [1, 2])
def test_split_z_inverse_equals_combined(lib, n, precision, tol, truncate, split):
    """The z inverse pass with w = k^2 a in its own one-region kernel (1), or
    as one one-region kernel that reads its input columns again per output
    line (2), gives the result of the combined three-region kernel."""
    import gturbo3d_gb300 as g
    gp, _ = configs(n, precision=precision, forcing="3d3c", truncate=truncate)
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=15)
    with g.Simulation(gp) as a, g.Simulation(gp) as b:
        a.set_state(b0)
        b.set_state(b0)
        a.set_tuning("z_split", split)
        b.set_tuning("z_split", 0)
        a.step(3, 5)
        b.step(3, 5)
        assert relerr(a.get_state(), b.get_state()) < tol
