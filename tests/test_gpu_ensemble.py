"""Ensemble runner (graph-captured and eager) against independent
simulations, and the launch-shape autotuner with its cache."""
import numpy as np
import pytest

from _helpers import configs, initial, relerr

pytestmark = pytest.mark.gpu


def _members():
    import gturbo3d_gb300 as g
    specs = [((16, 16, 16), "fp64", 3.0, 2e-3), ((32, 32, 32), "fp64", 7.0, 1e-3),
             ((32, 16, 8), "fp64", 1.5, 5e-3), ((32, 32, 32), "mixed", 12.0, 1e-3),
             ((16, 16, 16), "mixed", 19.0, 3e-3)]
    params, states = [], []
    for k, (n, prec, om, nu) in enumerate(specs):
        gp, _ = configs(n, precision=prec, forcing="3d3c", omega=om, nu=nu, dt=2e-3)
        gp.famp = g.forcing_amplitude(0.1, gp)
        params.append(gp)
        states.append(initial(n, seed=20 + k))
    return params, states


@pytest.mark.parametrize("graph", [True, False])
def test_ensemble_matches_individual_runs(lib, graph):
    import gturbo3d_gb300 as g
    params, states = _members()
    seeds = np.arange(100, 100 + len(params), dtype=np.int32)
    nsteps = 70                                  # crosses the 64-step forcing chunk
    refs, rseeds = [], []
    for p, b, s in zip(params, states, seeds):
        with g.Simulation(p) as sim:
            sim.set_state(b)
            rseeds.append(sim.step(nsteps, int(s)))
            refs.append(sim.get_state())
    with g.api.Ensemble(params) as ens:
        for i, b in enumerate(states):
            ens.set_state(i, b)
        out_seeds = ens.step(nsteps, seeds, graph=graph)
        assert list(out_seeds) == rseeds
        for i in range(len(params)):
            got = ens.get_state(i)
            assert relerr(got, refs[i]) < 1e-14, i
        e = ens.energy()
    assert np.all(np.isfinite(e)) and np.all(e > 0)


def test_ensemble_graph_equals_eager_bitwise(lib):
    import gturbo3d_gb300 as g
    params, states = _members()
    seeds = np.arange(7, 7 + len(params), dtype=np.int32)
    res = []
    for graph in (True, False):
        with g.api.Ensemble(params) as ens:
            for i, b in enumerate(states):
                ens.set_state(i, b)
            ens.step(5, seeds, graph=graph)
            res.append([ens.get_state(i) for i in range(len(params))])
    for a, b in zip(*res):
        for c in range(3):
            assert np.array_equal(a[c], b[c])


def test_autotune_and_cache(lib, tmp_path):
    import gturbo3d_gb300 as g
    gp, _ = configs(64, precision="mixed", forcing="3d3c")
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(64, seed=31)
    cache = str(tmp_path / "tuning.jsonl")
    with g.Simulation(gp) as tuned, g.Simulation(gp) as plain:
        tuned.set_state(b0)
        plain.set_state(b0)
        before = tuned.get_state()
        ms = g.api.autotune(tuned, cache)
        assert ms > 0
        assert relerr(tuned.get_state(), before) == 0.0      # the state is restored
        assert g.api.autotune(tuned, cache) == -1.0           # now from the cache
        s1 = tuned.step(4, 5)
        s2 = plain.step(4, 5)
        assert s1 == s2
        assert relerr(tuned.get_state(), plain.get_state()) < 1e-6
    text = open(cache).read()
    assert '"key": "64x64x64/mixed/pruned/' in text


def _class_members():
    """Three grid classes of two or more members (different Omega, nu, dt,
    forcing kind and forcing count within a class) and two lone members."""
    import gturbo3d_gb300 as g
    specs = [((32, 32, 32), "mixed", "3d3c", 3.0, 1e-3, 2e-3), ((32, 32, 32), "mixed", "3d3c", 11.0, 2e-3, 3e-3),
             ((32, 32, 32), "mixed", "2d2c", 17.0, 5e-4, 1e-3), ((32, 16, 8), "fp64", "3d3c", 2.0, 1e-3, 2e-3),
             ((32, 16, 8), "fp64", "none", 9.0, 3e-3, 4e-3), ((16, 16, 16), "fp64", "3d3c", 5.0, 1e-3, 2e-3),
             ((64, 32, 16), "mixed", "3d3c", 4.0, 1e-3, 2e-3), ((16, 16, 16), "mixed", "3d3c", 6.0, 1e-3, 2e-3),
             ((16, 16, 16), "mixed", "3d3c", 7.0, 2e-3, 1e-3)]
    params, states = [], []
    for k, (n, prec, forcing, om, nu, dt) in enumerate(specs):
        gp, _ = configs(n, precision=prec, forcing=forcing, omega=om, nu=nu, dt=dt)
        if forcing != "none":
            gp.famp = g.forcing_amplitude(0.1, gp)
        params.append(gp)
        states.append(initial(n, seed=40 + k))
    return params, states


def test_ensemble_grid_classes(lib):
    import gturbo3d_gb300 as g
    params, _ = _class_members()
    with g.api.Ensemble(params) as ens:
        cls = ens.classes()
    assert cls[0] == cls[1] == cls[2] >= 0
    assert cls[3] == cls[4] >= 0 and cls[3] != cls[0]
    assert cls[7] == cls[8] >= 0 and cls[7] not in (cls[0], cls[3])
    assert cls[5] == -1 and cls[6] == -1


@pytest.mark.parametrize("graph", [True, False])
@pytest.mark.parametrize("batching", [True, False])
def test_batched_classes_match_individual_runs(lib, graph, batching):
    """Members advanced by one launch per pass for their grid class give the
    states and seeds of the same members stepped one by one (70 steps: a
    64-step graph chunk and a shorter direct one)."""
    import gturbo3d_gb300 as g
    params, states = _class_members()
    seeds = np.arange(300, 300 + len(params), dtype=np.int32)
    nsteps = 70
    refs, rseeds = [], []
    for p, b, s in zip(params, states, seeds):
        with g.Simulation(p) as sim:
            sim.set_state(b)
            rseeds.append(sim.step(nsteps, int(s)) if p.forcing else (sim.step(nsteps), int(s))[1])
            refs.append(sim.get_state())
    with g.api.Ensemble(params) as ens:
        ens.set_batching(batching)
        for i, b in enumerate(states):
            ens.set_state(i, b)
        out_seeds = ens.step(nsteps, seeds, graph=graph)
        assert list(out_seeds) == rseeds
        for i in range(len(params)):
            assert relerr(ens.get_state(i), refs[i]) < 1e-14, i


def test_batched_class_with_a_member_off_the_kept_set(lib):
    """A class whose members disagree on the pruned path runs member by
    member for that call and still matches the individual runs."""
    import gturbo3d_gb300 as g
    params, states = _class_members()
    params, states = params[:3], states[:3]
    bad = [x.copy() for x in states[1]]
    bad[0][0, 0, 16] = 1e-4                     # kx = NX/2: outside the kept set
    states[1] = bad
    seeds = np.arange(5, 8, dtype=np.int32)
    refs = []
    for p, b, s in zip(params, states, seeds):
        with g.Simulation(p) as sim:
            sim.set_state(b)
            sim.step(6, int(s))
            refs.append(sim.get_state())
    with g.api.Ensemble(params) as ens:
        for i, b in enumerate(states):
            ens.set_state(i, b)
        ens.step(6, seeds, graph=False)
        for i in range(3):
            assert relerr(ens.get_state(i), refs[i]) < 1e-14, i


def test_batched_cluster_pair_z_pass_matches_individual_runs(lib):
    """Mixed members with 1024-point z columns run the z forward pass on
    thread-block cluster pairs by default; one batched launch per pass for
    their class (the member on a spare grid axis of the cluster launch) gives
    the states of the members stepped one by one."""
    import gturbo3d_gb300 as g
    n = (16, 16, 1024)
    params, states = [], []
    for k in range(3):
        gp, _ = configs(n, precision="mixed", forcing="3d3c", omega=2.0 + k, nu=1e-3 * (1 + k))
        gp.famp = g.forcing_amplitude(0.1, gp)
        params.append(gp)
        states.append(initial(n, seed=70 + k))
    with g.Simulation(params[0]) as sim:
        assert sim.get_tuning("z_cluster") == 1
    seeds = np.arange(11, 14, dtype=np.int32)
    refs = []
    for p, b, s in zip(params, states, seeds):
        with g.Simulation(p) as sim:
            sim.set_state(b)
            sim.step(5, int(s))
            refs.append(sim.get_state())
    with g.api.Ensemble(params) as ens:
        cls = ens.classes()
        assert cls[0] == cls[1] == cls[2] >= 0
        for i, b in enumerate(states):
            ens.set_state(i, b)
        ens.step(5, seeds, graph=False)
        for i in range(3):
            assert relerr(ens.get_state(i), refs[i]) < 1e-14, i
