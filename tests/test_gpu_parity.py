"""GPU pair loop through the C ABI vs the reference (golden fixtures) and the
oracle: integer counts bit-identical, weighted sums within 1e-6."""
import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import Golden, check_sums, golden_names

pytestmark = pytest.mark.gpu


def _ctx_for(p, S, D, tuning=None):
    cats = host.prepare(p, [("S", S), ("D", D)])
    ctx = _lib.Context(p)
    if tuning:
        ctx.set_tuning(*tuning)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    return ctx


@pytest.mark.parametrize("engine", ["fast", "fp64", "cell_fp64"])
@pytest.mark.parametrize("name", golden_names())
def test_matches_reference_golden(name, engine):
    g = Golden(name)
    ctx = _ctx_for(g.params, g.S, g.D)
    r = ctx.count("SD", 0, 1, engine=engine)
    assert r["n_binned"] == g.n_in
    assert r["n_window"] == g.n_total
    assert np.array_equal(r["num"], g.raw_num)
    check_sums(r["sums"], g.raw_sums, label=f"{name}/{engine}")


@pytest.mark.parametrize("tuning", [(1, 0, 0), (3, 0, 0), (2, 9, 0)])
def test_tuning_variants_match(tuning):
    """Cell size and block-local Pi window change the work split, not the result."""
    g = Golden("box_wpp_uniform")
    ctx = _ctx_for(g.params, g.S, g.D, tuning)
    r = ctx.count("SD", 0, 1)
    assert np.array_equal(r["num"], g.raw_num)
    check_sums(r["sums"], g.raw_sums, label=str(tuning))


def test_large_box_matches_oracle():
    """The 20,000-point uniform box (wgg, 8 cubes) in full."""
    wl = synth.box_uniform_wgg()
    p = wl.params
    ocats = oracle.read_like_reference(p, [("S", wl.shape), ("D", wl.density)])
    num, sums, n_total, n_in = oracle.port_corels2(p, "SD", ocats["D"], ocats["S"])
    ctx = _ctx_for(p, wl.shape, wl.density)
    r = ctx.count("SD", 0, 1)
    assert r["n_binned"] == n_in and r["n_window"] == n_total
    assert np.array_equal(r["num"], num)
    check_sums(r["sums"], sums)


@pytest.mark.parametrize("name", ["box_lattice_edges", "box_wgg_uniform", "box_wpp_uniform",
                                  "box_linear_bins_nojk"])
def test_twin_counts_match_reference_golden(name):
    """Cross terms whose S and D samples read the same file (wgg, w++; an
    integer lattice with pairs exactly on bin edges; linear bins with self
    pairs): the twin count -- each unordered pair tested once, both orders
    added -- equals the reference, and so does the count of every order."""
    g = Golden(name)
    ctx = _ctx_for(g.params, g.S, g.D)
    for twin in (True, False):
        ctx.set_twin(twin)
        r = ctx.count("SD", 0, 1)
        assert ctx.last_twin() == twin, name
        assert (r["n_binned"], r["n_window"]) == (g.n_in, g.n_total), (name, twin)
        assert np.array_equal(r["num"], g.raw_num), (name, twin)
        check_sums(r["sums"], g.raw_sums, label=f"{name} twin={twin}")
    ctx.close()


def test_twin_clustered_wpp_matches_oracle():
    """A clustered periodic w++ box with 27 cubes, S = D read twice (the
    jackknife keep flags differ between the reads): the twin count equals the
    oracle's corels2 over every row, and a row sample (no twin) still does."""
    c = synth.neyman_scott(300, 80.0, 3.0, 300.0, 71, nside_jk=3)
    p = synth._box_params(which_corr=2, L=300.0, rmin=0.1, rmax=50.0, nrp=20, npi=40,
                          pmax=80.0, njk=27, n=c.n)
    ocats = oracle.read_like_reference(p, [("S", c), ("D", c)])
    num, sums, n_total, n_in = oracle.port_corels2(p, "SD", ocats["D"], ocats["S"])
    ctx = _ctx_for(p, c, c)
    r = ctx.count("SD", 0, 1)
    assert ctx.last_twin()
    assert (r["n_binned"], r["n_window"]) == (n_in, n_total)
    assert np.array_equal(r["num"], num)
    check_sums(r["sums"], sums, label="twin")
    rs = ctx.count("SD", 0, 1, row_stride=7, row_offset=2)
    assert not ctx.last_twin()
    ref = oracle.port_corels2(p, "SD", ocats["D"], ocats["S"], row_stride=7, row_offset=2)
    assert np.array_equal(rs["num"], ref[0])
    check_sums(rs["sums"], ref[1], label="row sample")
    ctx.close()


def test_clustered_shapes_row_subsample_matches_oracle():
    """The 200,000-galaxy clustered wg+ box on every 97th outer row."""
    wl = synth.box_ns_wgp()
    p = wl.params
    ocats = oracle.read_like_reference(p, [("S", wl.shape), ("D", wl.density)])
    ref = oracle.port_corels2(p, "SD", ocats["D"], ocats["S"], row_stride=97, row_offset=5)
    ctx = _ctx_for(p, wl.shape, wl.density)
    for eng in ("fast", "fp64"):
        r = ctx.count("SD", 0, 1, engine=eng, row_stride=97, row_offset=5)
        assert r["n_binned"] == ref[3] and r["n_window"] == ref[2]
        assert np.array_equal(r["num"], ref[0])
        check_sums(r["sums"], ref[1], label=eng)


def test_full_clustered_box_fast_equals_fp64():
    """Full 200k box: the mixed-precision kernel equals the plain FP64 kernel."""
    wl = synth.box_ns_wgp()
    ctx = _ctx_for(wl.params, wl.shape, wl.density)
    a = ctx.count("SD", 0, 1, engine="fast")
    b = ctx.count("SD", 0, 1, engine="fp64")
    assert a["n_binned"] == b["n_binned"] and a["n_window"] == b["n_window"]
    assert np.array_equal(a["num"], b["num"])
    check_sums(a["sums"], b["sums"])


def test_repeat_is_deterministic_in_counts():
    g = Golden("box_wgp_clustered")
    ctx = _ctx_for(g.params, g.S, g.D)
    a = ctx.count("SD", 0, 1)
    b = ctx.count("SD", 0, 1)
    assert np.array_equal(a["num"], b["num"])
    assert np.allclose(a["sums"], b["sums"], rtol=1e-12, atol=1e-12 * np.abs(a["sums"]).max())


def test_batch_of_boxes_matches_individual_counts():
    """Several uneven sub-boxes in one persistent launch (cpc_count_batch)."""
    wls = synth.box_batch_wpp(n_boxes=6, seed=3, scale=0.02)
    ctxs = []
    for w in wls:
        ctxs.append(_ctx_for(w.params, w.shape, w.density))
    rs = _lib.count_batch([(c, "SD", 0, 1) for c in ctxs])
    for w, c, r in zip(wls, ctxs, rs):
        ocats = oracle.read_like_reference(w.params, [("S", w.shape), ("D", w.density)])
        num, sums, n_total, n_in = oracle.port_corels2(w.params, "SD", ocats["D"], ocats["S"])
        assert r["n_binned"] == n_in and r["n_window"] == n_total
        assert np.array_equal(r["num"], num)
        check_sums(r["sums"], sums)


def test_empty_catalogue_counts_nothing():
    p = synth.box_uniform_wgg().params
    e = synth.Catalog(np.zeros(0), np.zeros(0), np.zeros(0), None, None, None, np.zeros(0, np.int32))
    c = synth.uniform_box(100, p.periodic_box_size, 1, nside_jk=2)
    ctx = _ctx_for(p, c, e)
    r = ctx.count("SD", 0, 1)
    assert r["n_binned"] == 0 and r["n_window"] == 0 and r["num"].sum() == 0


def test_bad_inputs_are_rejected_with_status():
    p = synth.box_uniform_wgg().params
    ctx = _lib.Context(p)
    c = synth.uniform_box(50, p.periodic_box_size, 2, nside_jk=2)
    bad = synth.Catalog(c.x.copy(), c.y, c.z, None, None, None, c.jk.copy())
    bad.jk[3] = 99
    with pytest.raises(_lib.CpcError) as e:
        ctx.upload(0, bad)
    assert e.value.status == 6  # CPC_ERR_RANGE
    nan = synth.Catalog(c.x.copy(), c.y, c.z, None, None, None, c.jk)
    nan.x[0] = np.nan
    with pytest.raises(_lib.CpcError) as e:
        ctx.upload(0, nan)
    assert e.value.status == 6
    with pytest.raises(_lib.CpcError) as e:
        ctx.count("SD", 0, 1)
    assert e.value.status == 5  # CPC_ERR_STATE: count before upload


def test_autotune_keeps_results_identical():
    """The autotuner rebuilds the cell lists on the device for several cell
    widths and Pi windows, keeps the fastest; the counts stay the reference's."""
    g = Golden("box_wgp_clustered")
    p = g.params
    cats = host.prepare(p, [("S", g.S), ("D", g.D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    k, w = ctx.autotune("SD", 0, 1, sample_stride=2)
    assert k in (2, 3, 4, 5, 6) and 0 <= w <= p.n_p_bin
    r = ctx.count("SD", 0, 1)
    assert r["n_binned"] == g.n_in and r["n_window"] == g.n_total
    assert np.array_equal(r["num"], g.raw_num)
    check_sums(r["sums"], g.raw_sums)
    # a later upload uses the tuned grid and pairs with the rebuilt slot
    ctx.upload(0, cats["D"])
    r2 = ctx.count("SD", 0, 1)
    assert np.array_equal(r2["num"], g.raw_num)
    ctx.close()


def test_autotune_rmu_tunes_cells_only():
    """r-mu binning (coordinates 7): the autotuner picks a cell width and
    leaves the mu window automatic (0); the counts stay the reference's."""
    g = Golden("box_ed_rmu")
    p = g.params
    cats = host.prepare(p, [("S", g.S), ("D", g.D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    k, w = ctx.autotune("SD", 0, 1, sample_stride=2)
    assert k in (2, 3, 4, 5, 6) and w == 0
    r = ctx.count("SD", 0, 1)
    assert r["n_binned"] == g.n_in and r["n_window"] == g.n_total
    assert np.array_equal(r["num"], g.raw_num)
    check_sums(r["sums"], g.raw_sums)
    ctx.close()


@pytest.mark.parametrize("engine", ["fast", "fp64"])
def test_async_count_on_a_caller_stream(engine):
    """cpc_count_async after work queued on a caller stream equals cpc_count;
    other calls are refused until cpc_count_finish."""
    import torch
    g = Golden("box_wgp_clustered")
    p = g.params
    cats = host.prepare(p, [("S", g.S), ("D", g.D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    ref = ctx.count("SD", 0, 1, engine=engine)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        junk = torch.ones(1 << 20, device="cuda")
        junk = junk * 2.0  # work queued before the count
    ctx.count_async("SD", 0, 1, engine=engine, stream=s.cuda_stream)
    with pytest.raises(_lib.CpcError):
        ctx.count("SD", 0, 1)
    r = ctx.finish()
    s.synchronize()
    assert r["n_binned"] == ref["n_binned"] == g.n_in and r["n_window"] == ref["n_window"]
    assert np.array_equal(r["num"], ref["num"])
    check_sums(r["sums"], g.raw_sums)
    with pytest.raises(_lib.CpcError):
        ctx.finish()  # nothing pending
    ctx.close()
