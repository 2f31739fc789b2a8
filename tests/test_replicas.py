"""Replicas-only multi-GPU logic on CPU with two gloo ranks: the shards of independent meshes
are disjoint and cover all of them, and the throughput reduction takes the slowest rank's time
and the sum of the units."""
import os

import pytest

from meshoptimizer_gb300 import replicas


def test_shard_partitions():
    items = list(range(37))
    parts = [replicas.shard(items, r, 4) for r in range(4)]
    flat = sorted(x for p in parts for x in p)
    assert flat == items
    assert all(set(a).isdisjoint(b) for i, a in enumerate(parts) for b in parts[i + 1:])
    with pytest.raises(ValueError):
        replicas.shard(items, 4, 4)


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replicas.shard(list(range(100)), rank, world)
    seconds = 1.0 + rank  # rank 1 is the slowest
    rate, sec, units = replicas.aggregate(seconds, float(len(mine)), dist=dist)
    q.put((rank, sorted(mine), rate, sec, units))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, s0, r0, t0, u0), (_, s1, r1, t1, u1) = out
    assert sorted(s0 + s1) == list(range(100)) and not set(s0) & set(s1)
    assert t0 == t1 == 2.0 and u0 == u1 == 100.0 and r0 == r1 == 50.0
