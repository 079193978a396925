"""The kernels the benchmarks time, checked against the oracle.

The 512^3 and 1024^3 benchmark grids run the passes instantiated for 512- and
1024-point lines (the default x pass for the mixed form at NX = 512 is the
parking form, x_fused = 3).  Those instantiations are exercised here on grids
that are long along one or two axes and short along the others, so that the
oracle (nlt.f90:16-89, produ.f90:9-101, trunc.f90:10-28, rkstep.f90:30-48 and
86-104, forcing_3d3c.f90:26-72) finishes in seconds: the library's default
tuning, each non-default tuning knob, and the 256^3 2D2C configuration.
Tolerances: FP64 1e-12 (one step) and 1e-11 (ten steps) relative L2 of the
state; mixed 1e-5.
"""
import os

import numpy as np
import pytest

from _helpers import configs, initial, relerr

pytestmark = pytest.mark.gpu

TOL = {("fp64", 1): 1e-12, ("fp64", 3): 1e-11, ("fp64", 10): 1e-11,
       ("mixed", 1): 1e-5, ("mixed", 3): 1e-5, ("mixed", 10): 1e-5}

_cache = {}


def _oracle(n, forcing, dt2, nsteps, seed, init_seed, threads=1, **phys):
    """(state, seed) of the oracle after nsteps, memoised per configuration."""
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle
    key = (n, forcing, dt2, nsteps, seed, init_seed, tuple(sorted(phys.items())))
    if key not in _cache:
        gp, op = configs(n, forcing=forcing, dt2_mode=dt2, **phys)
        if forcing != "none":
            op.famp = g.forcing_amplitude(0.1, gp)
        orc = Oracle(op, threads=threads)
        _cache[key] = orc.run(initial(n, seed=init_seed), seed, nsteps)
    return _cache[key]


def _library(n, precision, forcing, dt2, nsteps, seed, init_seed, tuning=None, pruning=True, **phys):
    import gturbo3d_gb300 as g
    gp, _ = configs(n, precision=precision, forcing=forcing, dt2_mode=dt2, **phys)
    if forcing != "none":
        gp.famp = g.forcing_amplitude(0.1, gp)
    with g.Simulation(gp) as sim:
        for k, v in (tuning or {}).items():
            sim.set_tuning(k, v)
        sim.set_pruning(pruning)
        sim.set_state(initial(n, seed=init_seed))
        s = sim.step(nsteps, seed)
        return sim.get_state(), s


LONG_LINES = [(512, 16, 16), (16, 512, 16), (16, 16, 512), (1024, 16, 8), (8, 1024, 16), (16, 8, 1024)]


@pytest.mark.parametrize("n", LONG_LINES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nsteps", [1, 10])
def test_default_passes_on_long_lines(lib, n, precision, nsteps):
    """512- and 1024-point x, y and z lines through the default passes (3D3C
    forcing, dt2 = dt/2) against the oracle."""
    ref, sref = _oracle(n, "3d3c", "rk2", nsteps, 8299396, 3)
    got, s = _library(n, precision, "3d3c", "rk2", nsteps, 8299396, 3)
    assert s == sref
    assert relerr(got, ref) < TOL[(precision, nsteps)]


def test_bench_default_x_pass_is_the_one_checked(lib):
    """The mixed form at NX = 512 defaults to the parking x pass (x_fused =
    3), FP64 and other line lengths to x_fused = 2: the forms the long-line
    cases above run."""
    import gturbo3d_gb300 as g
    for n, prec, want in [((512, 16, 16), "mixed", 3), ((512, 16, 16), "fp64", 2),
                          ((1024, 16, 8), "mixed", 2), ((16, 512, 16), "mixed", 2)]:
        gp, _ = configs(n, precision=prec)
        with g.Simulation(gp) as sim:
            assert sim.get_tuning("x_fused") == want, (n, prec)
            assert sim.get_tuning("fuse_stage") == 0 and sim.get_tuning("z_split") == 0
    # the cluster-pair z forward pass is the default only for mixed z columns of 1024 points
    for n, prec, want in [((16, 8, 1024), "mixed", 1), ((16, 8, 1024), "fp64", 0),
                          ((16, 16, 512), "mixed", 0)]:
        gp, _ = configs(n, precision=prec)
        with g.Simulation(gp) as sim:
            assert sim.get_tuning("z_cluster") == want, (n, prec)
    # TMA-loaded z tiles: the forward (bit 1) and inverse (bit 2) passes for mixed z
    # columns of 256 and 512 points, the inverse pass's tensor stores (bit 4) at 256
    for n, prec, want in [((16, 16, 512), "mixed", 3), ((16, 16, 512), "fp64", 0),
                          ((16, 16, 256), "mixed", 7), ((16, 16, 128), "mixed", 0), ((16, 8, 1024), "mixed", 0)]:
        gp, _ = configs(n, precision=prec)
        with g.Simulation(gp) as sim:
            assert sim.get_tuning("z_tma") == want, (n, prec)


@pytest.mark.parametrize("n", [(512, 512, 16), (16, 512, 512), (512, 16, 512)])
def test_default_passes_two_long_axes_mixed(lib, n):
    """Two 512-point axes at once (the tile lists and grids of the 512^3
    launch along those axes), mixed form, two steps."""
    ref, sref = _oracle(n, "3d3c", "rk2", 2, 12345, 4, threads=os.cpu_count() or 1)
    got, s = _library(n, "mixed", "3d3c", "rk2", 2, 12345, 4)
    assert s == sref
    assert relerr(got, ref) < 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_as_built_dt2_on_512_lines(lib, precision):
    """The as-built scheme (dt2 = 0, N1 discarded) through the 512-point passes."""
    n = (512, 16, 16)
    ref, sref = _oracle(n, "3d3c", "as_built", 10, 77, 5)
    got, s = _library(n, precision, "3d3c", "as_built", 10, 77, 5)
    assert s == sref
    assert relerr(got, ref) < TOL[(precision, 10)]


VARIANTS = [dict(x_fused=0), dict(x_fused=1), dict(x_fused=2), dict(x_fused=3), dict(fuse_stage=1),
            dict(z_split=1), dict(z_split=2), dict(z_split=3), dict(z_split=3, z_tx=4), dict(y_pairs=0), dict(y_tx=4, z_tx=4), dict(y_tx=16, z_tx=16),
            dict(fuse_stage=1, z_tx=4, y_tx=2), dict(y_prefetch=0), dict(y_prefetch=2),
            dict(y_prefetch=2, y_tx=4), dict(y_prefetch=2, y_pairs=0), dict(overlap=1),
            dict(overlap=1, fuse_stage=1), dict(overlap=1, y_prefetch=0, z_tx=4), dict(slab_pipe=1),
            dict(slab_pipe=1, y_prefetch=0, x_fused=2), dict(zf_pipe=1), dict(zf_pipe=1, z_tx=4),
            dict(zf_pipe=1, z_split=3), dict(z_cluster=1), dict(z_cluster=1, fuse_stage=1),
            dict(z_cluster=1, y_prefetch=0, x_fused=2), dict(z_cluster=1, zf_pipe=1), dict(z_tma=1),
            dict(z_tma=1, fuse_stage=1), dict(z_tma=0), dict(z_tma=2), dict(z_tma=3), dict(z_tma=3, z_tx=4),
            dict(z_tma=6), dict(z_tma=7), dict(z_tma=7, fuse_stage=1), dict(z_tma=7, y_prefetch=0)]


@pytest.mark.parametrize("tuning", VARIANTS, ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
@pytest.mark.parametrize("n,precision", [((64, 32, 32), "fp64"), ((64, 32, 32), "mixed"),
                                         ((512, 16, 16), "mixed"), ((16, 16, 512), "mixed"),
                                         ((16, 16, 256), "mixed"), ((16, 512, 16), "fp64")])
def test_every_tuning_knob_against_the_oracle(lib, tuning, n, precision):
    """Each non-default launch shape checked against the oracle itself (not
    against another shape of the library), three steps."""
    ref, sref = _oracle(n, "3d3c", "rk2", 3, 4242, 6)
    got, s = _library(n, precision, "3d3c", "rk2", 3, 4242, 6, tuning=tuning)
    assert s == sref
    assert relerr(got, ref) < TOL[(precision, 3)]


@pytest.mark.parametrize("n,precision", [((512, 16, 16), "mixed"), ((16, 16, 512), "fp64"), ((64, 32, 32), "mixed")])
def test_unpruned_passes_against_the_oracle(lib, n, precision):
    """The full (unpruned) passes, forced with gt_set_pruning(0)."""
    ref, sref = _oracle(n, "3d3c", "rk2", 3, 4242, 6)
    got, s = _library(n, precision, "3d3c", "rk2", 3, 4242, 6, pruning=False)
    assert s == sref
    assert relerr(got, ref) < TOL[(precision, 3)]


@pytest.fixture(scope="module")
def config2_reference():
    """The 256^3 2D2C configuration (nu = 5e-4, Omega = 10, dt = 2e-3, seed 1,
    injection 0.1 on 2 <= |k_h| <= 3): the oracle's state and glob after
    three steps."""
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import Oracle, glob
    from gturbo3d_gb300.workloads import precision_params
    n = 256
    gp = precision_params("fp64", n)
    _, op = configs(n, forcing="2d2c", nu=5e-4, omega=10.0, dt=2e-3)
    op.famp = gp.famp
    orc = Oracle(op, threads=os.cpu_count() or 1)
    b0 = initial(n, seed=1)
    ref, sref = orc.run(b0, 1, 3)
    return b0, ref, sref, glob(ref, op, orc.wk)


@pytest.mark.slow
@pytest.mark.parametrize("precision,tol,dtol", [("fp64", 1e-11, 1e-11), ("mixed", 1e-5, 1e-5)])
def test_config2_256cubed_2d2c_against_the_oracle(lib, config2_reference, precision, tol, dtol):
    """Configuration 2 at full size for three steps: state and the energy /
    dissipation terms of glob (diagnostics.f90:126-153) against the oracle."""
    import gturbo3d_gb300 as g
    from gturbo3d_gb300.workloads import precision_params
    b0, ref, sref, gref = config2_reference
    with g.Simulation(precision_params(precision, 256)) as sim:
        sim.set_state(b0)
        s = sim.step(3, 1)
        got = sim.get_state()
        d = sim.glob()
    assert s == sref
    assert relerr(got, ref) < tol
    e_ref = np.asarray(gref["energy"])
    assert np.max(np.abs(d["energy"][:6] - e_ref[:6]) / np.abs(e_ref[:6])) < dtol
