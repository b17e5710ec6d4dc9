"""Replicas over the GPUs of one node: one process per GPU, each integrating its own disks.

The path has no data exchange between disks, so N GPUs run N independent shares of the
work (weak scaling: a fixed share per rank) and the only collectives are the timing ones:
the maximum of the ranks' timed regions and the sum of their simulated years.  These
helpers take an initialised ``torch.distributed`` module (or ``None`` for one process); the
tensors live on ``device`` (CPU for gloo, the rank's GPU for NCCL).
"""
from __future__ import annotations


def shard(items, rank, world):
    """The rank's contiguous share of ``items`` (sizes differ by at most one)."""
    items = list(items)
    n = len(items)
    lo = (n * rank) // world
    hi = (n * (rank + 1)) // world
    return items[lo:hi]


def _reduce(value, dist, op, device):
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value, dist, device="cpu"):
    """The largest ``value`` over the ranks (the whole job's timed region)."""
    return _reduce(value, dist, None if dist is None else dist.ReduceOp.MAX, device)


def sum_over_ranks(value, dist, device="cpu"):
    """The sum of ``value`` over the ranks (work done by the whole job)."""
    return _reduce(value, dist, None if dist is None else dist.ReduceOp.SUM, device)


def job_rate(local_units, local_seconds, dist, device="cpu"):
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    units = sum_over_ranks(local_units, dist, device)
    secs = max_over_ranks(local_seconds, dist, device)
    return units / secs if secs > 0 else float("nan"), units, secs
