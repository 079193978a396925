"""Tangent-linear and adjoint RK2 step: the TL/adjoint dot-product test,
finite differences of the plain forward, the checkpointed gradient, the
mixed form against the FP64 gradient, and a torch.autograd.Function harness
(test-only) built on gt_gradient."""
import numpy as np
import pytest

from _helpers import configs, initial, relerr

pytestmark = pytest.mark.gpu


def inner(x, y):
    """<x, y> = sum w Re(conj x y), w = 1 on the kx = 0 and kx = N/2 planes, 2 elsewhere."""
    tot = 0.0
    for a, b in zip(x, y):
        w = np.full(a.shape[-1], 2.0)
        w[0] = 1.0
        w[-1] = 1.0
        tot += float(np.sum(w * (np.conj(a) * b).real))
    return tot


def real_field_spectrum(shape, seed, p):
    """A random spectral field that is the transform of a real field."""
    from oracle.gturbo_oracle import fft_dir
    rng = np.random.default_rng(seed)
    nz, ny, nh = shape
    nx = 2 * (nh - 1)
    return [fft_dir(rng.standard_normal((nz, ny, nx)), p) for _ in range(3)]


@pytest.mark.parametrize("n,phys", [((16, 16, 16), {}), ((32, 16, 8), dict(omega=3.0)), ((16, 16, 16), dict(truncate=0))])
@pytest.mark.parametrize("dt2", ["rk2", "as_built"])
def test_dot_product(lib, n, phys, dt2):
    import gturbo3d_gb300 as g
    gp, op = configs(n, forcing="none", dt2_mode=dt2, **phys)
    b0 = initial(n, seed=3)
    with g.Simulation(gp) as sim:
        sim.set_state(b0)
        x = real_field_spectrum(sim.shape, 1, op)
        y = real_field_spectrum(sim.shape, 2, op)
        lhs = inner(y, sim.tl_step(x))
        rhs = inner(sim.adj_step(y), x)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), abs(rhs))


def test_tl_against_central_differences(lib):
    import gturbo3d_gb300 as g
    n = (16, 16, 16)
    gp, op = configs(n, forcing="3d3c", omega=4.0)
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=4)
    with g.Simulation(gp) as sim:
        sim.set_state(b0)
        d = real_field_spectrum(sim.shape, 5, op)
        scale = np.sqrt(inner(b0, b0) / inner(d, d))
        d = [scale * x for x in d]
        tl = sim.tl_step(d)
        h = 1e-5
        out = []
        for sgn in (+1, -1):
            sim.set_state([b + sgn * h * x for b, x in zip(b0, d)])
            sim.step(1, 77)                      # same forcing both ways: it cancels
            out.append(sim.get_state())
        fd = [(a - b) / (2 * h) for a, b in zip(*out)]
    assert relerr(tl, fd) < 1e-8


@pytest.mark.parametrize("precision", ["fp64"])
def test_gradient_against_finite_differences(lib, precision):
    """dJ along random directions: adjoint gradient vs central differences
    (h = 1e-6 relative), 16^3, 12 steps, checkpoints every 5 steps."""
    import gturbo3d_gb300 as g
    n = (16, 16, 16)
    gp, op = configs(n, precision=precision, forcing="3d3c", nu=1e-3, omega=5.0, dt=4e-3)
    gp.famp = g.forcing_amplitude(0.1, gp)
    b0 = initial(n, seed=3)
    nsteps, K, kmin, seed = 12, 5, 4.0, 3
    with g.Simulation(gp) as sim:
        sim.set_state(b0)
        J, grad = sim.gradient(nsteps, seed, K, kmin)
        assert relerr(sim.get_state(), b0) == 0.0     # state restored

        def Jof(b):
            sim.set_state(b)
            sim.step(nsteps, seed)
            return sim.objective(kmin)

        assert abs(Jof(b0) - J) <= 1e-12 * abs(J)
        errs = []
        for k in range(3):
            d = real_field_spectrum(sim.shape, 10 + k, op)
            d = [x * np.sqrt(inner(b0, b0) / inner(d, d)) for x in d]
            h = 1e-6
            fd = (Jof([b + h * x for b, x in zip(b0, d)]) - Jof([b - h * x for b, x in zip(b0, d)])) / (2 * h)
            ad = inner(grad, d)
            errs.append(abs(fd - ad) / max(abs(fd), 1e-300))
    assert max(errs) < 1e-6, errs


def test_mixed_gradient_against_fp64(lib):
    import gturbo3d_gb300 as g
    n = (16, 16, 16)
    grads = {}
    for prec in ("fp64", "mixed"):
        gp, _ = configs(n, precision=prec, forcing="3d3c", nu=1e-3, omega=5.0, dt=4e-3)
        gp.famp = g.forcing_amplitude(0.1, gp)
        with g.Simulation(gp) as sim:
            sim.set_state(initial(n, seed=3))
            grads[prec] = sim.gradient(10, 3, 5, 4.0)
    assert abs(grads["mixed"][0] - grads["fp64"][0]) / grads["fp64"][0] < 1e-4
    assert relerr(grads["mixed"][1], grads["fp64"][1]) < 1e-3


def test_torch_autograd_harness(lib):
    """A test-only torch.autograd.Function whose backward is gt_gradient:
    gradcheck-style directional derivative against central differences."""
    torch = pytest.importorskip("torch")
    import gturbo3d_gb300 as g
    n = (16, 16, 16)
    gp, op = configs(n, forcing="3d3c", nu=1e-3, omega=5.0, dt=4e-3)
    gp.famp = g.forcing_amplitude(0.1, gp)
    sim = g.Simulation(gp)
    shape = sim.shape
    nsteps, K, kmin, seed = 6, 3, 4.0, 3

    def to_np(t):
        a = t.detach().cpu().numpy()
        return [np.ascontiguousarray(a[c]).view(np.complex128).reshape(shape) for c in range(3)]

    class ShellEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, b):
            sim.set_state(to_np(b))
            J, gr = sim.gradient(nsteps, seed, K, kmin)
            w = np.full(shape[-1], 2.0)
            w[0] = w[-1] = 1.0
            # dJ = sum w Re(conj(g) db) = sum over the real view of (w g) . db
            gv = np.stack([(x * w).view(np.float64).reshape(shape[0], shape[1], -1) for x in gr])
            ctx.save_for_backward(torch.from_numpy(gv))
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            (gv,) = ctx.saved_tensors
            return gout * gv

    b0 = initial(n, seed=3)
    bt = torch.from_numpy(np.stack([x.view(np.float64).reshape(shape[0], shape[1], -1) for x in b0]))
    bt.requires_grad_(True)
    J = ShellEnergy.apply(bt)
    J.backward()
    d = torch.from_numpy(np.stack([x.view(np.float64).reshape(shape[0], shape[1], -1)
                                   for x in real_field_spectrum(shape, 9, op)]))
    d = d * (bt.detach().norm() / d.norm())
    h = 1e-6

    def Jval(b):
        sim.set_state(to_np(b))
        sim.step(nsteps, seed)
        return sim.objective(kmin)

    fd = (Jval(bt.detach() + h * d) - Jval(bt.detach() - h * d)) / (2 * h)
    ad = float((bt.grad * d).sum())
    sim.close()
    assert abs(fd - ad) / abs(fd) < 1e-6
