"""Two processes (gloo, CPU) each count half of the outer rows and reduce the
raw blocks: the sum equals the single-process count.  The per-rank counter
here is the oracle, so the test runs without a GPU; on GPUs each rank counts
its shard of the fast engine's work units (cpc_set_shard) or, for the sky and
FP64 engines, the same (row_stride, row_offset) of rows -- the GPU test
test_gpu_graph.py::test_unit_shards_sum_to_the_whole_count covers the unit
shards on one GPU."""
import os
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    import oracle
    from corr_pc_gb300 import parallel
    from helpers import Golden
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = Golden("box_wgp_clustered")
    cats = oracle.read_like_reference(g.params, [("S", g.S), ("D", g.D)])
    stride, off = parallel.shard(rank, world)
    num, sums, n_total, n_in = oracle.port_corels2(g.params, "SD", cats["D"], cats["S"],
                                                   n_threads=1, row_stride=stride, row_offset=off)
    cnt = np.array([n_total, n_in], dtype=np.int64)
    parallel.reduce_blocks(num, sums, cnt)
    if rank == 0:
        q.put((num, sums, cnt))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_row_sharding_reduces_to_full_count():
    from helpers import Golden
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    num, sums, cnt = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    g = Golden("box_wgp_clustered")
    assert np.array_equal(num, g.raw_num)
    assert cnt[1] == g.n_in and cnt[0] == g.n_total
    scale = np.abs(g.raw_sums).max(axis=(0, 1, 2)) + 1e-300
    assert (np.abs(sums - g.raw_sums) / scale).max() < 1e-12
