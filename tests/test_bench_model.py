"""The algorithmic-byte model behind bench.py's roofline figures: its kept-mode
and active-column counts follow the reference's truncation rule (the oracle's
trunc mask, trunc.f90:14-28), and the 512^3 per-step total is the figure the
roofline reports."""
import numpy as np
import pytest


@pytest.mark.parametrize("n", [16, 32, 64])
def test_kept_modes_and_columns_follow_trunc(n):
    import bench
    from oracle import gturbo_oracle as O

    wk = O.defk(O.Params(nx=n, ny=n, nz=n))
    keep = ~O.trunc_mask(wk)                       # [nz, ny, nh]; the origin is zeroed too
    pb = bench.pass_bytes(n, "mixed", pruned=True)
    # recover K, A, xa from the per-pass formulas: zinv = (3K + 6An) e, yfwd = (3 xa n^2 + 3An) e,
    # xcross = 9 xa n^2 e (e = 8 bytes per FP32 complex value)
    e = 8
    xa = pb["xcross"] // (9 * n * n * e)
    A = (pb["yfwd"] // e - 3 * xa * n * n) // (3 * n)
    K = (pb["zinv_curl"] // e - 6 * A * n) // 3
    assert K == int(keep.sum()) + 1                # + the (0,0,0) mode, kept in the byte count
    assert A == int(keep.any(axis=0).sum())        # (kx, ky) columns with a kept mode
    assert xa == int(keep.any(axis=(0, 1)).sum())  # kx planes with a kept mode


def test_step_bytes_at_512():
    """21.19 GB per pruned step at 512^3; without pruning the fused-pass model's
    90 field-sized transfers per step."""
    import bench
    pb = bench.pass_bytes(512, "mixed", pruned=True)
    step = 2 * sum(pb[k] for k in ("zinv_curl", "yinv", "xcross", "yfwd", "zfwd_epilogue"))
    assert step == 21189284784
    full = bench.pass_bytes(512, "mixed", pruned=False)
    assert 2 * sum(full[k] for k in ("zinv_curl", "yinv", "xcross", "yfwd", "zfwd_epilogue")) == 90 * full["field_bytes"]
