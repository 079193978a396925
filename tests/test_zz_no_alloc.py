"""gt_energy_noalloc: the kinetic energy for callers that cannot allocate
device memory (their arrays belong to another runtime, e.g. an OpenACC data
region, and cudaMalloc is off limits in their time loop).  The entry point
works on the caller's own device arrays and stream, with a fixed scratch
array inside the library.  Its result must equal gt_energy's (FP64
tolerance of these tests, 1e-12 relative) on consecutive calls, whose
scratch contents are left over from the call before.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import math

import numpy as np
import pytest

from _helpers import configs, initial

pytestmark = pytest.mark.gpu


def _gt_energy(g, gp, b):
    with g.Simulation(gp) as sim:
        sim.set_state(b)
        e = np.zeros(3)
        g._lib.check(sim.lib.gt_energy(sim.h, e.ctypes.data_as(g.api.C.POINTER(g.api.C.c_double))),
                     "gt_energy")
    return e


def test_energy_noalloc_matches_gt_energy(lib):
    torch = pytest.importorskip("torch")
    import gturbo3d_gb300 as g
    nx, ny, nz = 32, 16, 64
    gp, _ = configs((nx, ny, nz), forcing="none")          # FP64 handle: the existing entry point
    b1 = initial((nx, ny, nz), seed=3)
    b2 = [2.0 * x + 0.1 * np.roll(x, 1, axis=0) for x in initial((nx, ny, nz), seed=4)]
    two_pi = 2 * math.pi
    # The test allocates the caller-owned device arrays; the entry point itself allocates nothing.
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for b in (b1, b2):                                      # two calls in a row
        ref = _gt_energy(g, gp, b)
        dev = [torch.from_numpy(np.ascontiguousarray(x).view(np.float64).copy()).to("cuda") for x in b]
        out.fill_(float("nan"))
        rc = lib.gt_energy_noalloc(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), nx, ny, nz,
                                   two_pi, two_pi, two_pi, out.data_ptr(), stream)
        assert rc == 0, lib.gt_last_error().decode()
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12)


def test_energy_noalloc_rejects_oversized_grid(lib):
    torch = pytest.importorskip("torch")
    from gturbo3d_gb300 import _lib
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    # 1024 x 1024 rows exceed the fixed scratch: rejected before any device work
    rc = lib.gt_energy_noalloc(p, p, p, 64, 1024, 1024, 6.28, 6.28, 6.28, p, None)
    assert rc == _lib.GT_EINVAL
    assert "exceeds the fixed scratch" in lib.gt_last_error().decode()
