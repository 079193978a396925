"""The N > 1 path's host logic on CPU ranks (gloo, world size 2): replicas
need no data-path collective; only the timing max and a gather of results."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from gturbo3d_gb300.replicas import gather_rows, max_over_ranks, replica_seed, shard_members
        sizes = [64] * 48 + [128] * 12 + [256] * 4
        mine = shard_members(sizes, world)[rank]
        rows = [[float(i), float(replica_seed(100, i))] for i in mine]
        allrows = gather_rows(rows, dist)
        tmax = max_over_ranks(1.5 + rank, dist)
        q.put((rank, sorted(int(r[0]) for r in allrows), tmax, replica_seed(2, rank)))
    finally:
        dist.destroy_process_group()


def test_replicas_two_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, members, tmax, seed in res:
        assert members == list(range(64))      # every member exactly once, gathered on all ranks
        assert tmax == 2.5                     # max over ranks
        assert seed == 2 + rank


def test_shard_balance():
    from gturbo3d_gb300.replicas import member_cost, shard_members
    sizes = [64] * 48 + [128] * 12 + [256] * 4
    for world in (1, 2, 4, 8):
        parts = shard_members(sizes, world)
        assert sorted(i for p in parts for i in p) == list(range(len(sizes)))
        loads = [sum(member_cost(sizes[i]) for i in p) for p in parts]
        biggest = max(member_cost(n) for n in sizes)
        assert max(loads) <= max(1.35 * (sum(loads) / world), biggest * 1.01)
