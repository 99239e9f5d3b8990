"""CUDA-graph replay of the fast box engine: a count captured once and
replayed gives the reference's results on every replay, a change of the launch
shape captures again, and direct launches give the same results."""
import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import Golden, check_sums

pytestmark = pytest.mark.gpu


def _ctx_for(p, S, D):
    cats = host.prepare(p, [("S", S), ("D", D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    return ctx


def _check(r, g, label):
    assert r["n_binned"] == g.n_in and r["n_window"] == g.n_total
    assert np.array_equal(r["num"], g.raw_num)
    check_sums(r["sums"], g.raw_sums, label=label)


@pytest.mark.parametrize("name", ["box_wgp_clustered", "box_wpp_weighted_distinct"])
def test_replayed_counts_match_reference(name):
    g = Golden(name)
    ctx = _ctx_for(g.params, g.S, g.D)
    for k in range(3):
        _check(ctx.count("SD", 0, 1), g, f"{name} replay {k}")
    captures, replays = ctx.graph_stats()
    assert captures == 1 and replays == 3
    # direct launches: the same results
    ctx.set_graph_replay(False)
    _check(ctx.count("SD", 0, 1), g, f"{name} direct")
    assert ctx.graph_stats() == (1, 3)


def test_changed_launch_shape_captures_again():
    g = Golden("box_wpp_uniform")
    ctx = _ctx_for(g.params, g.S, g.D)
    # S and D read the same file: counted in every order here (a twin count
    # takes other units than a row sample; it is checked at the end)
    ctx.set_twin(False)
    _check(ctx.count("SD", 0, 1), g, "first")
    ctx.set_tuning(0, 9, 0)  # another Pi window: other units, grid, shared memory
    _check(ctx.count("SD", 0, 1), g, "window 9")
    _check(ctx.count("SD", 0, 1), g, "window 9 replay")
    assert ctx.graph_stats() == (2, 3)
    # a row sample differs only in the job descriptor (copied in before each
    # replay): the same graph serves it and the full count after it
    r = ctx.count("SD", 0, 1, row_stride=5, row_offset=2)
    assert 0 < r["n_binned"] < g.n_in
    _check(ctx.count("SD", 0, 1), g, "full again")
    assert ctx.graph_stats() == (2, 5)
    # the twin count (each unordered pair once, both orders added) runs other
    # units and shared memory: a capture of its own, the reference's results
    ctx.set_twin(True)
    _check(ctx.count("SD", 0, 1), g, "twin")
    assert ctx.last_twin() and ctx.graph_stats() == (3, 6)


def test_async_count_replays_on_a_caller_stream():
    import torch
    g = Golden("box_wgp_clustered")
    ctx = _ctx_for(g.params, g.S, g.D)
    s = torch.cuda.Stream()
    for _ in range(2):
        ctx.count_async("SD", 0, 1, stream=s.cuda_stream)
        _check(ctx.finish(), g, "async")
    assert ctx.graph_stats() == (1, 2)


def test_batch_replays_match_oracle():
    wls = synth.box_batch_wpp(n_boxes=5, seed=11, scale=0.02)
    ctxs = [_ctx_for(w.params, w.shape, w.density) for w in wls]
    ref = []
    for w in wls:
        oc = oracle.read_like_reference(w.params, [("S", w.shape), ("D", w.density)])
        ref.append(oracle.port_corels2(w.params, "SD", oc["D"], oc["S"]))
    for rep in range(2):
        rs = _lib.count_batch([(c, "SD", 0, 1) for c in ctxs])
        for r, (num, sums, n_total, n_in) in zip(rs, ref):
            assert r["n_binned"] == n_in and r["n_window"] == n_total
            assert np.array_equal(r["num"], num)
            check_sums(r["sums"], sums, label=f"batch replay {rep}")
    assert ctxs[0].graph_stats() == (1, 2)


def test_new_scales_capture_again():
    """The fixed-point scales are kernel parameters: catalogues with other
    ellipticity bounds must not replay a graph made for the old ones."""
    g = Golden("box_wgp_clustered")
    ctx = _ctx_for(g.params, g.S, g.D)
    _check(ctx.count("SD", 0, 1), g, "first")
    half = lambda c: synth.Catalog(c.x, c.y, c.z, c.w,
                                   None if c.e1 is None else 0.37 * np.asarray(c.e1),
                                   None if c.e2 is None else 0.37 * np.asarray(c.e2), c.jk, c.e3)
    S2, D2 = half(g.S), half(g.D)
    cats = host.prepare(g.params, [("S", S2), ("D", D2)])
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    r = ctx.count("SD", 0, 1)
    assert ctx.graph_stats()[0] == 2
    oc = oracle.read_like_reference(g.params, [("S", S2), ("D", D2)])
    num, sums, n_total, n_in = oracle.port_corels2(g.params, "SD", oc["D"], oc["S"])
    assert r["n_binned"] == n_in and r["n_window"] == n_total
    assert np.array_equal(r["num"], num)
    check_sums(r["sums"], sums, label="scaled shapes")


def test_edge_queue_growth_counts_again(monkeypatch):
    """A context that starts with a 16-entry edge queue overflows it, grows it,
    counts again (a new graph) and still gives the reference's results."""
    g = Golden("box_lattice_edges")
    monkeypatch.setenv("CPC_EDGE_QUEUE_INIT", "16")
    ctx = _ctx_for(g.params, g.S, g.D)
    r = ctx.count("SD", 0, 1)
    assert r["n_rechecked"] > 16
    _check(r, g, "grown queue")
    _check(ctx.count("SD", 0, 1), g, "grown queue, replay")


@pytest.mark.parametrize("name", ["box_wgp_clustered", "box_wpp_weighted_distinct"])
def test_unit_shards_sum_to_the_whole_count(name):
    """Three contexts, each counting one shard of the work units (as three GPUs
    would): the raw blocks add up to the reference's."""
    g = Golden(name)
    parts = []
    for sh in range(3):
        ctx = _ctx_for(g.params, g.S, g.D)
        ctx.set_shard(sh, 3)
        parts.append(ctx.count("SD", 0, 1))
        ctx.close()
    assert all(0 < p["n_binned"] < g.n_in for p in parts)
    assert sum(p["n_binned"] for p in parts) == g.n_in
    assert sum(p["n_window"] for p in parts) == g.n_total
    assert np.array_equal(sum(p["num"] for p in parts), g.raw_num)
    check_sums(sum(p["sums"] for p in parts), g.raw_sums, label=f"{name} shards")


def test_bad_shard_is_rejected():
    g = Golden("box_wgp_clustered")
    ctx = _ctx_for(g.params, g.S, g.D)
    with pytest.raises(_lib.CpcError):
        ctx.set_shard(3, 3)
    with pytest.raises(_lib.CpcError):
        ctx.set_shard(0, 0)


@pytest.mark.parametrize("name", ["auto_box_wpp_rebin", "auto_box_wgp_unsorted"])
def test_unit_shards_of_auto_pairs_sum_to_the_reference(name):
    """corels1 (cpc_count_auto) on two work-unit shards adds up to the
    reference's auto-correlation block."""
    from helpers import AutoGolden
    g = AutoGolden(name)
    rnum, rsums, rin, rtot = g.term("SS")
    cats = host.prepare(g.params, g.read_order(), table=g.table)
    parts = []
    for sh in range(2):
        ctx = _lib.Context(g.params, table=g.table)
        ctx.upload(0, cats["S"])
        ctx.set_shard(sh, 2)
        parts.append(ctx.count_auto("SS", 0))
        ctx.close()
    assert sum(p["n_binned"] for p in parts) == rin
    assert sum(p["n_window"] for p in parts) == rtot
    assert np.array_equal(sum(p["num"] for p in parts), rnum)
    check_sums(sum(p["sums"] for p in parts), rsums, label=f"{name} auto shards")


def test_unit_shards_of_a_batch_sum_to_the_whole_batch():
    """Every context of a batch on the same shard of its units, then the other
    shard: the two batches add up to the oracle's counts of every box."""
    wls = synth.box_batch_wpp(n_boxes=4, seed=5, scale=0.02)
    ref = []
    for w in wls:
        oc = oracle.read_like_reference(w.params, [("S", w.shape), ("D", w.density)])
        ref.append(oracle.port_corels2(w.params, "SD", oc["D"], oc["S"]))
    ctxs = [_ctx_for(w.params, w.shape, w.density) for w in wls]
    halves = []
    for sh in range(2):
        for c in ctxs:
            c.set_shard(sh, 2)
        halves.append(_lib.count_batch([(c, "SD", 0, 1) for c in ctxs]))
    for k, (num, sums, n_total, n_in) in enumerate(ref):
        a, b = halves[0][k], halves[1][k]
        assert a["n_binned"] + b["n_binned"] == n_in
        assert a["n_window"] + b["n_window"] == n_total
        assert np.array_equal(a["num"] + b["num"], num)
        check_sums(a["sums"] + b["sums"], sums, label=f"batch box {k} shards")
