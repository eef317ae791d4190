"""Replicas on several GPUs (one process per GPU): the path does not shard a table, so independent
units (observables, thresholds, batched instances, requests) are split across ranks with no
collective on the data path; only the report combines the ranks (slowest rank's time, total work).
"""
from __future__ import annotations


def shard(items, rank, world):
    """The contiguous share of `items` of one rank (sizes differ by at most one)."""
    items = list(items)
    n, world = len(items), max(1, int(world))
    lo = rank * n // world
    hi = (rank + 1) * n // world
    return items[lo:hi]


def aggregate(ms, work, device=None):
    """(max ms over ranks, total work over ranks); the identity without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms), float(work)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(w)
    return float(t.item()), float(w.item())
