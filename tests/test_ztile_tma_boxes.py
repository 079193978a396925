"""Invariants of the TMA boxes of the z inverse pass, checked on the CPU against the
oracle's truncation mask (trunc.f90:14-28).

The kernel (k_zinv_tma, csrc/gt_kernels_impl.cuh) loads, for a tile of 16 columns
X = 16 tile .. 16 tile + 15 of row y, the z-rows [0, hend) and [tstart, nz) in boxes
of 32 rows, with hend = min(nz, (zc / 32 + 1) 32) and
tstart = max(hend, (nz - zc) / 32 * 32).  zc comes from the host (upload_tables,
csrc/gt_capi.cu): the largest z <= nz/2 whose row keeps the tile's first column,
with the kept prefix xcut[z][y] of each row.  Restated here, the boxes must cover
every kept row of every column of the tile, lie inside [0, nz), not overlap, and add
up to the transaction bytes the kernel expects.
"""
import numpy as np
import pytest

from _helpers import configs

BOX = 32
TX = 16


def _xcut(n):
    from oracle.gturbo_oracle import Oracle, trunc_mask
    _, op = configs(n)
    m = trunc_mask(Oracle(op).wk)     # [nz][ny][nh], True = zeroed
    m[0, 0, 0] = False                # the (0,0,0) mode is a point, not part of the row prefix
    nz, ny, nh = m.shape
    kept = ~m
    # kept prefix per row: kx < xcut[z][y] (the trunc sum grows with kx^2)
    xcut = np.where(kept.all(axis=2), nh, np.argmin(kept, axis=2))
    assert np.array_equal(kept, np.arange(nh)[None, None, :] < xcut[:, :, None])
    return xcut, kept


def _tiles(xcut):
    nz, ny = xcut.shape
    out = []
    for y in range(ny):
        for t in range(0, (xcut[0, y] + TX - 1) // TX):
            X = t * TX
            z = 0
            while z + 1 <= nz // 2 and xcut[z + 1, y] > X:
                z += 1
            out.append((t, y, z))
    return out


@pytest.mark.parametrize("n", [(32, 32, 64), (64, 32, 128), (32, 16, 256), (128, 64, 64)])
def test_boxes_cover_the_kept_rows_of_every_tile_column(n):
    xcut, kept = _xcut(n)
    nz, ny = xcut.shape
    nh = kept.shape[2]
    for t, y, zc in _tiles(xcut):
        hend = min(nz, (zc // BOX + 1) * BOX)
        tstart = max(hend, (nz - zc) // BOX * BOX)
        rows = set(range(0, hend)) | set(range(tstart, nz))
        nbox = hend // BOX + (nz - tstart) // BOX
        assert 0 < hend <= nz and hend <= tstart <= nz
        assert hend % BOX == 0 and tstart % BOX == 0 and (nz - tstart) % BOX == 0
        assert len(rows) == nbox * BOX                 # no overlap; expect_tx = nbox boxes
        for X in range(t * TX, min(nh, t * TX + TX)):
            for z in np.nonzero(kept[:, y, X])[0]:
                assert z in rows, (t, y, X, z)


def test_kept_rows_are_a_symmetric_interval_in_kz():
    """The premise of zc: for each (kx, ky) the kept z form |kz| <= some bound
    (the trunc sum grows with kz^2), so z <= zc and z >= nz - zc."""
    xcut, kept = _xcut((32, 32, 64))
    nz = xcut.shape[0]
    kz = np.where(np.arange(nz) <= nz // 2, np.arange(nz), np.arange(nz) - nz)
    for y in range(xcut.shape[1]):
        for X in range(kept.shape[2]):
            zs = np.nonzero(kept[:, y, X])[0]
            if len(zs):
                bound = np.abs(kz[zs]).max()
                assert set(zs) == set(np.nonzero(np.abs(kz) <= bound)[0])


@pytest.mark.parametrize("lnx", [4, 5, 6, 7, 8, 9, 10])
@pytest.mark.parametrize("lnz", [4, 5, 6, 7, 8, 9])
def test_tensor_copies_meet_the_alignment_rules(lnx, lnz):
    """The tensor maps and boxes of both TMA z passes (tensor_maps_zcols and the
    launches in csrc/gt_kernels_impl.cuh), restated for FP32 rows padded to
    nhp = nh rounded up to 16 complex values: the innermost coordinate of every
    copy, the strides and the box's inner extent are multiples of 16 bytes, every
    box lies inside the padded row, every shared destination is 128-byte aligned,
    and the shared tile plus its mbarriers fits the 227 KB opt-in."""
    csize = 8                                   # FP32 complex
    nx, nz = 1 << lnx, 1 << lnz
    nh = nx // 2 + 1
    align = 128 // csize
    nhp = (nh + align - 1) // align * align
    dims_x = 2 * nhp                            # floats
    stride_row, stride_plane = nhp * 8, 32 * nhp * 8
    assert stride_row % 16 == 0 and stride_plane % 16 == 0
    box_x = 32                                  # floats: 16 complex columns
    assert box_x * 4 % 16 == 0
    for tile in range((nh + TX - 1) // TX):
        x = tile * 2 * TX                       # floats
        assert x * 4 % 16 == 0
        assert x + box_x <= dims_x              # whole box inside the padded row
    # z forward pass: boxes of min(nz, 256) rows at z = 0, 256, ...; region f at f * nz * 16 columns
    zbox = min(nz, 256)
    for f in range(3):
        for h in range(nz // zbox):
            assert ((f * nz + h * zbox) * TX * csize) % 128 == 0
    assert 3 * nz * TX * csize + 3 * 8 <= 227 * 1024
    # z inverse pass (nz >= 32): boxes of 32 rows, regions of nz rows of 8 column pairs (16 bytes each)
    if nz >= BOX:
        for c in range(3):
            for z0 in range(0, nz, BOX):
                assert ((c * nz * (TX // 2) + z0 * (TX // 2)) * 16) % 128 == 0
        assert 3 * nz * TX * csize + 6 * 8 <= 227 * 1024
        # its tensor stores (z_tma bit 4): boxes of min(nz, 256) rows from each region,
        # at non-negative coordinates, covering the region's rows once
        obox = min(nz, 256)
        for c in range(3):
            starts = list(range(0, nz, obox))
            assert sum(obox for _ in starts) == nz and min(starts) >= 0
            for z0 in starts:
                assert ((c * nz * (TX // 2) + z0 * (TX // 2)) * 16) % 128 == 0
