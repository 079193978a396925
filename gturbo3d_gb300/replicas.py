"""Host logic of the multi-GPU path: independent replicas, one per rank.

A single field does not shard into independent units (every 3D FFT would need
all-to-all transposes), so N GPUs run N independent simulations: replica r
uses forcing/initial-field seed ``base + r``.  Ensemble members (the batched
configuration: 48 x 64^3 + 12 x 128^3 + 4 x 256^3) are spread over ranks by
cost with a deterministic greedy assignment.  The only collectives are on the
host side of the measurement (a barrier and a max of the timed interval) and
the gather of per-member diagnostics.
"""
from __future__ import annotations

import math


def replica_seed(base: int, rank: int) -> int:
    return base + rank


def member_cost(n: int) -> float:
    """Relative cost of one RK2 step on an n^3 grid (FFT flops ~ n^3 log2 n^3)."""
    return n ** 3 * math.log2(n ** 3)


def shard_members(sizes: list[int], world: int) -> list[list[int]]:
    """Assigns member indices to ranks: largest first, each to the currently
    least-loaded rank (ties to the lowest rank).  Deterministic."""
    order = sorted(range(len(sizes)), key=lambda i: (-member_cost(sizes[i]), i))
    load = [0.0] * world
    out: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += member_cost(sizes[i])
    for r in range(world):
        out[r].sort()
    return out


def max_over_ranks(value: float, dist=None) -> float:
    """Max of a per-rank scalar (the timed interval) over all ranks."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    backend = dist.get_backend()
    dev = "cuda" if backend == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_rows(rows: list[list[float]], dist=None) -> list[list[float]]:
    """Gathers every rank's list of per-member result rows to all ranks, in
    rank order."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return rows
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, rows)
    return [r for part in out for r in part]
