"""Sharding of the pair loop over processes (one GPU each).

The work of one corels2 call splits without any exchange until the end; the
raw histogram blocks of the ranks are summed once (one reduction of int64
counts and FP64 sums).  Two ways to split it:

* the fast box engine shards its work units (cpc_set_shard): rank r of W counts
  the units i with i % W == r.  The units partition the pairs (tiles of outer
  rows against slices of their candidates), and each rank does about 1/W of the
  work;
* the sky kernels and the plain FP64 engine shard the outer rows (cpc_count's
  row_stride / row_offset: rows with original index i % W == r), which they
  skip at no cost.

Used with torch.distributed (NCCL between GPUs, gloo on CPU)."""
from __future__ import annotations

import numpy as np


def shard(rank: int, world: int) -> tuple[int, int]:
    """(row_stride, row_offset) of this rank's outer rows."""
    return (world, rank) if world > 1 else (1, 0)


def shard_context(ctx, rank: int, world: int, *, fast_box: bool = True) -> tuple[int, int]:
    """Set up this rank's share of the counts made on ctx: for the fast box
    engine the work-unit shard (returns row_stride 1, row_offset 0 for
    cpc_count), otherwise the (row_stride, row_offset) of its outer rows."""
    if fast_box:
        ctx.set_shard(rank, max(1, world))
        return 1, 0
    return shard(rank, world)


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
