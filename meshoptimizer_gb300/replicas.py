"""Multi-GPU form of the simplifier: replicas only.

One mesh does not shard: its greedy collapse order is global, so splitting it would change the
result. Independent meshes (cluster groups, requests) partition across ranks with no collective
on the data path; the only cross-rank step is the timing/throughput reduction at the end.
"""
from __future__ import annotations


def shard(items, rank: int, world: int):
    """Round-robin partition of independent units: rank r gets items r, r+world, ..."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    return items[rank::world]


def shard_indices(count: int, rank: int, world: int):
    return list(range(rank, count, world))


def aggregate(local_seconds: float, local_units: float, dist=None, device=None):
    """Whole-job throughput of independent replicas: units summed over ranks divided by the
    slowest rank's time (max over ranks). Without a process group, the local values."""
    if dist is None or not dist.is_initialized():
        return local_units / local_seconds if local_seconds > 0 else 0.0, local_seconds, local_units
    import torch

    t = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    u = torch.tensor([local_units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    seconds, units = float(t.item()), float(u.item())
    return (units / seconds if seconds > 0 else 0.0), seconds, units
