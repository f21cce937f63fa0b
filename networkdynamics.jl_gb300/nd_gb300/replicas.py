"""Independent replicas across processes (one per GPU).

A single network's RHS does not shard here (it would need a halo exchange per call that
the reference does not have), so several GPUs run replicas.  Ensembles and training-data
generation consist of independent instances: each rank takes a contiguous share of the
instances, and the host gathers the per-instance results in rank order.  No collective
touches the data path; the gather is a host-side object gather.
"""
from __future__ import annotations

import numpy as np


def shard(n: int, rank: int, world: int) -> range:
    """The contiguous range of instances rank `rank` of `world` takes (sizes differ by at most 1)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def gather_instances(local, world: int):
    """Concatenate per-rank arrays (leading axis = instances) in rank order on every rank."""
    if world == 1:
        return np.asarray(local)
    import torch.distributed as dist
    parts = [None] * world
    dist.all_gather_object(parts, np.asarray(local))
    return np.concatenate(parts, axis=0)


def max_over_ranks(x: float, world: int) -> float:
    """The largest of the ranks' values (timings are reported as the slowest rank's)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
