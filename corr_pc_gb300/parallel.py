"""Sharding of the pair loop over processes (one GPU each).

The outer rows of corels2 are independent: rank r of W counts the rows whose
original index i has i % W == r (cpc_count's row_stride/row_offset), and the
raw histogram blocks are summed once at the end -- one reduction of int64
counts and FP64 sums, no other exchange.  Used with torch.distributed (NCCL
between GPUs, gloo on CPU)."""
from __future__ import annotations

import numpy as np


def shard(rank: int, world: int) -> tuple[int, int]:
    """(row_stride, row_offset) of this rank's outer rows."""
    return (world, rank) if world > 1 else (1, 0)


def reduce_blocks(num: np.ndarray, sums: np.ndarray, counters: np.ndarray):
    """Sum the raw histogram blocks over all ranks (in place, every rank gets
    the total).  Counts travel as int64, sums as float64."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return num, sums, counters
    for a in (num, sums, counters):
        t = torch.from_numpy(a)
        dist.all_reduce(t)
    return num, sums, counters
