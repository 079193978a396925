"""3D transforms through the library's FFT passes against numpy (pocketfft),
the stand-in for cuFFT's D2Z / Z2D at the reference's fft_dir / fft_inv."""
import numpy as np
import pytest

from _helpers import configs, relerr

pytestmark = pytest.mark.gpu

SHAPES = [(8, 8, 8), (16, 16, 16), (32, 16, 8), (8, 32, 16), (64, 64, 64), (128, 32, 64),
          (16, 1024, 8), (1024, 8, 16)]


@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("precision,tol", [("fp64", 2e-15), ("mixed", 2e-7)])
def test_fft_dir_inv_vs_numpy(lib, n, precision, tol):
    import gturbo3d_gb300 as g
    from oracle.gturbo_oracle import fft_dir, fft_inv
    gp, op = configs(n, precision=precision, forcing="none")
    rng = np.random.default_rng(1)
    x = rng.standard_normal((op.nz, op.ny, op.nx))
    with g.Simulation(gp) as sim:
        X = sim.fft_dir(x)
        Xr = fft_dir(x, op)
        assert relerr([X], [Xr]) < tol * np.log2(x.size)
        y = sim.fft_inv(Xr)
        yr = fft_inv(Xr, op)
        assert relerr([y], [yr]) < tol * np.log2(x.size)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-14), ("mixed", 1e-6)])
def test_single_mode_known_answer(lib, precision, tol):
    """A single Fourier mode (kx,ky,kz) = (3,-2,5) of amplitude A inverts to
    A e^{i k.x} + c.c. on the grid (the unnormalised C2R of fft_inv.f90)."""
    import gturbo3d_gb300 as g
    gp, op = configs((16, 32, 16), precision=precision, forcing="none")
    z = np.zeros((16, 32, 9), np.complex128)
    A = 0.75 - 0.4j
    z[5, 32 - 2, 3] = A
    with g.Simulation(gp) as sim:
        x = sim.fft_inv(z)
    zz, yy, xx = np.meshgrid(np.arange(16), np.arange(32), np.arange(16), indexing="ij")
    ph = 2 * np.pi * (3 * xx / 16 - 2 * yy / 32 + 5 * zz / 16)
    ref = 2 * (A.real * np.cos(ph) - A.imag * np.sin(ph))
    assert np.max(np.abs(x - ref)) < tol * 4


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-14), ("mixed", 1e-6)])
def test_round_trip_512(lib, precision, tol):
    """fft_dir(fft_inv(X)) == X at the benchmark size 512^3 (a size-independent
    property checked at full size)."""
    import gturbo3d_gb300 as g
    gp, op = configs(512, precision=precision, forcing="none")
    rng = np.random.default_rng(2)
    x = rng.standard_normal((512, 512, 512))
    with g.Simulation(gp) as sim:
        X = sim.fft_dir(x)
        y = sim.fft_inv(X)
    assert relerr([y], [x]) < tol * 30
