"""Event sharding across ranks (one GPU per rank).

Solves are independent given the slowness, so ranks take disjoint
contiguous blocks of solves and run them with no communication; an
inversion then sums the per-rank FP64 gradients and misfits with one
all-reduce per evaluation (the reference sums with mpi_sum over
station-strided ranks, scripts/inversion.jl:36-39,124).
"""
from __future__ import annotations

import numpy as np


def shard_solves(n_solves: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of the contiguous block of solves owned by `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_solves, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def allreduce_sum_f64(arrays, group=None):
    """Sum FP64 arrays (misfit, gradients) over ranks with torch.distributed."""
    import torch
    import torch.distributed as dist

    flat = np.concatenate([np.asarray(a, np.float64).ravel() for a in arrays])
    t = torch.from_numpy(flat)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    out, off = [], 0
    for a in arrays:
        a = np.asarray(a)
        out.append(t[off:off + a.size].numpy().reshape(a.shape))
        off += a.size
    return out
