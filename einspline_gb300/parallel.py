"""Sharding of the evaluation across ranks (one process per GPU).

The path needs no collective on its data: splines are independent (a table
too large for one GPU is split along the spline axis, each rank owning a
contiguous block of columns) and points are independent (walkers are split
across ranks that each hold a replica of the table).  The only
communication is the benchmark's timing: the slowest rank's time and the
total work.
"""
from __future__ import annotations


def shard_range(n: int, rank: int, world: int):
    """Contiguous block [lo, hi) of n items owned by rank (sizes differ by at
    most one, lower ranks take the remainder)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, rem = divmod(n, world)
    lo = rank * base + min(rank, rem)
    return lo, lo + base + (1 if rank < rem else 0)


def shard_splines(num_splines: int, rank: int, world: int, align: int = 32):
    """Spline columns [first, first+count) for rank when splitting a table
    along the spline axis, in blocks of `align` splines so that every shard's
    rows stay 128-byte aligned."""
    blocks = (num_splines + align - 1) // align
    lo, hi = shard_range(blocks, rank, world)
    first = lo * align
    return first, max(0, min(num_splines, hi * align) - first)


def aggregate(ms: float, work: float, device=None):
    """(max of ms over ranks, sum of work over ranks) with torch.distributed
    when it is initialised, else the local values."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms, work
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    w = torch.tensor([work], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())
