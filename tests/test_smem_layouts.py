"""Shared-memory layouts of the line transforms, checked on a model of the
shared-memory banks (32 banks of 4 bytes; an access of a warp is served in
128-byte phases, 16 threads for 8-byte elements and 8 for 16-byte ones, and a
phase takes as many wavefronts as the most distinct words any bank holds).

The index functions and the Stockham exchange patterns are restated from
gturbo3d_gb300/csrc/gt_fft.cuh (swz, StridedIdxLg, fft_stages_ct): stage s
with 2^LGNS points done and radix 2^LR stores element
((t >> LGNS) << (LGNS + LR)) + (t & (NS - 1)) + j NS, and every exchange
loads element t + i L/8 back.
"""
import pytest


def swz(e):
    return e ^ ((e >> 3) & 15)


def strided_idx(e, x, lg):
    return ((e + (e >> 3)) << lg) + x


def strided_rows(L):
    return L + (L >> 3)


def stages(L):
    lg, lgns, out = L.bit_length() - 1, 0, []
    while lg - lgns > 0:
        lr = min(3, lg - lgns)
        out.append((lgns, lr))
        lgns += lr
    return out


def stage_stores(L, t, lgns, lr):
    """Elements thread t stores after the stage (fft_stages_ct, radix 8/4/2)."""
    T, NS, out = L // 8, 1 << lgns, []
    groups = {3: 1, 2: 2, 1: 4}[lr]
    for m in range(groups):
        b = t + m * T
        base = ((b >> lgns) << (lgns + lr)) + (b & (NS - 1))
        out += [base + j * NS for j in range(1 << lr)]
    return out


def wavefronts(byte_addrs, esize):
    per_phase = 128 // esize
    wf = 0
    for p0 in range(0, len(byte_addrs), per_phase):
        banks = {}
        for a in byte_addrs[p0:p0 + per_phase]:
            for w in range(esize // 4):
                word = a // 4 + w
                banks.setdefault(word % 32, set()).add(word)
        wf += max(len(v) for v in banks.values())
    return wf, (len(byte_addrs) + per_phase - 1) // per_phase


def excess(L, esize, addr_of, nthreads):
    """Wavefronts over the minimum, summed over every exchange store and load
    of one transform; addr_of(thread, element) is the element's slot."""
    got = need = 0
    accesses = []
    for lgns, lr in stages(L)[:-1]:          # the last stage writes global memory
        for k in range(len(stage_stores(L, 0, lgns, lr))):
            accesses.append(lambda th, t, lgns=lgns, lr=lr, k=k: stage_stores(L, t, lgns, lr)[k])
    for i in range(8):
        accesses.append(lambda th, t, i=i: t + i * (L // 8))
    for acc in accesses:
        for w0 in range(0, max(nthreads, 32), 32):
            addrs = [addr_of(th, acc) * esize for th in range(w0, w0 + 32)]
            g, n = wavefronts(addrs, esize)
            got += g
            need += n
    return got / need


def x_line_addr(L, line_stride):
    """Slot of a thread's element in the x pass: groups of L/8 threads, one
    line each, lines line_stride elements apart, XOR-swizzled."""
    T = L // 8

    def addr(th, acc):
        g, t = divmod(th, T)
        return g * line_stride + swz(acc(th, t))
    return addr


def tile_addr(L, lgTP):
    """Slot of a thread's element in a y/z tile: TP = 2^lgTP columns (or
    column pairs) side by side, thread = t * TP + column."""
    TP = 1 << lgTP

    def addr(th, acc):
        x, t = th & (TP - 1), th >> lgTP
        return strided_idx(acc(th, t), x, lgTP)
    return addr


@pytest.mark.parametrize("L", [8, 16, 32, 64, 128, 256, 512, 1024])
def test_swizzle_is_a_permutation_of_each_line(L):
    """No two logical elements of a line share a slot, and the line needs no
    padding (the swizzle permutes aligned groups of 16)."""
    assert sorted(swz(e) for e in range(L)) == list(range(L))


@pytest.mark.parametrize("L", [8, 16, 64, 512, 1024])
@pytest.mark.parametrize("lg", [0, 1, 2, 3, 4])
def test_strided_tile_index_is_injective_and_in_bounds(L, lg):
    slots = {strided_idx(e, x, lg) for e in range(L) for x in range(1 << lg)}
    assert len(slots) == L << lg
    assert max(slots) < strided_rows(L) << lg


@pytest.mark.parametrize("L", [128, 256, 512, 1024])
@pytest.mark.parametrize("esize", [8, 16])
def test_x_lines_conflict_free_with_one_group_per_phase(L, esize):
    """x lines of 128 points or more (FP32 or FP64 complex; the CTrip planes of
    k_xbatch are 3 L apart): every exchange store and load of every stage
    takes the minimum number of wavefronts."""
    assert excess(L, esize, x_line_addr(L, 3 * L), 2 * (L // 8)) == 1.0


@pytest.mark.parametrize("L,esize,expect", [(64, 8, 2.0), (32, 8, 4.0), (16, 8, 8.0), (32, 16, 2.0)])
def test_x_lines_short_lines_share_banks_across_groups(L, esize, expect):
    """Lines of 64 points or fewer put several thread groups in one 128-byte
    phase, and their line bases (3 L elements apart, a multiple of 128 bytes)
    map to the same banks: the exchanges take `expect` times the minimum.
    Offsetting each group's base by L/8 more elements would remove it; the
    grids this affects (64^3 ensemble members and smaller) are launch- and
    latency-bound rather than shared-memory bound."""
    assert excess(L, esize, x_line_addr(L, 3 * L), 32) == expect
    padded = excess(L, esize, x_line_addr(L, 3 * L + L // 8), 32)
    assert padded == 1.0


@pytest.mark.parametrize("L", [64, 128, 256, 512, 1024])
@pytest.mark.parametrize("lgTP,esize", [(2, 16), (3, 8)])
def test_strided_tiles_conflict_free(L, lgTP, esize):
    """y/z tiles at the default widths: 4 column pairs of FP32 (16-byte
    elements) or FP64 columns, and 8 FP32 columns of the z forward pass."""
    assert excess(L, esize, tile_addr(L, lgTP), (L // 8) << lgTP) == 1.0


def dense_tile_addr(L, lgTP):
    """Slot of a thread's element in a dense z tile of the TMA-loaded passes
    (DenseIdxLg: e << lgTP | x, no padding rows)."""
    TP = 1 << lgTP

    def addr(th, acc):
        x, t = th & (TP - 1), th >> lgTP
        return (acc(th, t) << lgTP) + x
    return addr


@pytest.mark.parametrize("L", [64, 128, 256, 512])
@pytest.mark.parametrize("lgTP,esize", [(4, 8), (3, 16)])
def test_dense_16_column_tiles_conflict_free(L, lgTP, esize):
    """The dense tiles of the TMA-loaded z passes: 16 FP32 columns, one per
    thread (k_zfwd_tma) or in pairs (k_zinv_tma).  A row is one 128-byte line
    and a warp's access covers whole rows, so every exchange store and load
    takes the minimum number of wavefronts without padding rows."""
    assert excess(L, esize, dense_tile_addr(L, lgTP), (L // 8) << lgTP) == 1.0


@pytest.mark.parametrize("L", [64, 512])
def test_dense_8_column_tiles_would_conflict(L):
    """The same dense layout with 8 FP32 columns (64-byte rows) does take
    extra wavefronts in some exchange, which is why the dense tiles are used
    only at 16 columns and the narrower tiles keep their padding rows."""
    assert excess(L, 8, dense_tile_addr(L, 3), (L // 8) << 3) > 1.0
