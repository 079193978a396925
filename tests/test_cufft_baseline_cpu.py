"""The reference-style GPU baseline of bench.py (CufftStep: the reference's
unfused routine sequence with torch.fft) computes the oracle's RK2 step: run
here with torch on the CPU on small grids, against the FP64 oracle."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n,forcing", [(16, "3d3c"), ((32, 16, 8), "3d3c"), (16, "2d2c")])
def test_cufft_step_matches_oracle(n, forcing):
    import bench
    import gturbo3d_gb300 as g
    from gturbo3d_gb300.synth import initial_potential
    from oracle import gturbo_oracle as O

    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    p = g.make_params(nx, ny, nz, precision="fp64", forcing=forcing, nu=2e-3, omega=5.0, dt=5e-3)
    p.famp = g.forcing_amplitude(0.1, p)
    b0 = initial_potential(nx, ny, nz, 3)
    st = bench.CufftStep(p, torch, torch.float64, device=torch.device("cpu"))
    b = [torch.as_tensor(x) for x in b0]
    adds, s = st.draw(3, 3)
    for k in range(3):
        b = st.step(b, adds[k])
    op = O.Params(nx=nx, ny=ny, nz=nz, nu=p.nu, omega=p.omega, dt=p.dt, famp=p.famp, k1f=p.k1f,
                  k2f=p.k2f, forcing=forcing, dt2_mode="rk2")
    ob, oseed = O.Oracle(op).run([x.copy() for x in b0], 3, 3)
    assert s == oseed
    num = sum(float(np.sum(np.abs(b[i].numpy() - ob[i]) ** 2)) for i in range(3))
    den = sum(float(np.sum(np.abs(ob[i]) ** 2)) for i in range(3))
    assert math.sqrt(num / den) < 1e-13
