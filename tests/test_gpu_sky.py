"""Sky pair loop (coordinates 0) on the GPU against the reference and the oracle.

The golden runs hold the reference's own histograms for the four sky terms
(SRd, RsRd, SD, DRs); counts must be identical and sums within 1e-6.  The
reference's DRs term of a wg+ run crashes (shape rotation of randoms read
without ellipticities), so the fixtures hold it as a density-density count and
only its counts and weights are compared."""
import copy

import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import SkyGolden, check_sums, sky_golden_names

pytestmark = pytest.mark.gpu

SLOTS = {"S": 0, "Rs": 1, "D": 2, "Rd": 3}


def _context(p, table, cats):
    ctx = _lib.Context(p, table=table)
    for role, slot in SLOTS.items():
        ctx.upload(slot, cats[role])
    return ctx


@pytest.mark.parametrize("engine", ["fast", "fp64"])
@pytest.mark.parametrize("name", sky_golden_names())
def test_sky_matches_reference(name, engine):
    g = SkyGolden(name)
    p = g.params
    cats = host.prepare(p, g.read_order(), table=g.table)
    ctx = _context(p, g.table, cats)
    for t in g.terms:
        kind, a, b = SkyGolden.KIND[t]
        r = ctx.count(kind, SLOTS[a], SLOTS[b], engine=engine)
        rnum, rsums, rin, rtot = g.term(t)
        assert (r["n_binned"], r["n_window"]) == (rin, rtot), t
        assert np.array_equal(r["num"], rnum), t
        if t == "DRs" and g.meta["drs_as_wgg"]:
            check_sums(r["sums"][..., :1], rsums[..., :1], label=t)
        else:
            check_sums(r["sums"], rsums, label=t)
    ctx.close()


def test_sky_clamp_pairs_take_the_host_tier():
    """Twins at the clamp angle of dA_calc: their bins depend on the last bits
    of cos/acos, so the GPU hands them to the host tier; counts stay exact."""
    g = SkyGolden("sky_twins_clamp")
    cats = host.prepare(g.params, g.read_order(), table=g.table)
    ctx = _context(g.params, g.table, cats)
    r = ctx.count("SD", SLOTS["D"], SLOTS["S"])
    rnum, _, rin, _ = g.term("SD")
    assert r["n_rechecked"] > 0
    assert r["n_binned"] == rin and np.array_equal(r["num"], rnum)
    ctx.close()


def test_sky_wpp_matches_oracle():
    """A larger w++ sky run with weights and 16 jackknife regions, every term
    against the oracle restatement (counts exact, sums within 1e-6)."""
    p = synth._sky_params(which_corr=2, rmin=0.3, rmax=60.0, nrp=15, npi=30, pmax=60.0, njk=16)
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    d = synth.sky_patch(5000, 41, t, nside_jk=4, with_shapes=True, weights=True)
    r = synth.sky_patch(12000, 42, t, nside_jk=4)
    order = [("S", d), ("Rs", r), ("D", d), ("Rd", r)]
    cats = host.prepare(p, order, table=t)
    ctx = _context(p, t, cats)
    ocats = oracle.read_like_reference(p, order, table=t)
    zsep = synth.derived_z_sep(p, t)[0]
    for term, (kind, a, b) in SkyGolden.KIND.items():
        g = ctx.count(kind, SLOTS[a], SLOTS[b])
        num, sums, n_total, n_in = oracle.port_corels2(p, kind, ocats[a], ocats[b], H_z=t.H,
                                                       dA_z=t.transverse, z_sep_max=zsep)
        assert (g["n_binned"], g["n_window"]) == (n_in, n_total), term
        assert np.array_equal(g["num"], num), term
        check_sums(g["sums"], sums, label=term)
    ctx.close()


def test_sky_row_subsample_and_swap():
    """Row subsampling partitions the outer rows; a smaller g1 is swapped."""
    g = SkyGolden("sky_wgp_jk")
    p = g.params
    cats = host.prepare(p, g.read_order(), table=g.table)
    ctx = _context(p, g.table, cats)
    full = ctx.count("SRd", SLOTS["Rd"], SLOTS["S"])
    parts = [ctx.count("SRd", SLOTS["Rd"], SLOTS["S"], row_stride=3, row_offset=o)
             for o in range(3)]
    assert np.array_equal(sum(q["num"] for q in parts), full["num"])
    assert sum(q["n_window"] for q in parts) == full["n_window"]
    ctx.close()


def test_sky_rejects_bad_input():
    g = SkyGolden("sky_wgp_jk")
    p = g.params
    cats = host.prepare(p, g.read_order(), table=g.table)
    ctx = _lib.Context(p, table=g.table)
    bad = copy.copy(cats["S"])
    bad.z = bad.z.copy()
    bad.z[5] = p.z_max + 1.0
    with pytest.raises(_lib.CpcError):
        ctx.upload(0, bad)
    bad = copy.copy(cats["S"])
    bad.dc = None
    with pytest.raises(_lib.CpcError):
        ctx.upload(0, bad)
    with pytest.raises(ValueError):
        _lib.Context(p)
    ctx.close()


@pytest.mark.parametrize("name", ["sky_wgp_jk", "sky_wgg_distinct_wrap"])
def test_sky_terms_in_one_launch_match_reference(name):
    """The four terms of a sky run (SRd, RsRd, SD, DRs) counted in one launch of
    the fast kernel (cpc_count_batch on one context) equal the reference's."""
    g = SkyGolden(name)
    p = g.params
    cats = host.prepare(p, g.read_order(), table=g.table)
    ctx = _context(p, g.table, cats)
    l0 = ctx.launches()
    jobs = [(ctx, SkyGolden.KIND[t][0], SLOTS[SkyGolden.KIND[t][1]], SLOTS[SkyGolden.KIND[t][2]])
            for t in g.terms]
    rs = _lib.count_batch(jobs)
    # one pair kernel plus one fixed-point conversion per term
    assert ctx.launches() - l0 == 1 + len(g.terms)
    for t, r in zip(g.terms, rs):
        rnum, rsums, rin, rtot = g.term(t)
        assert (r["n_binned"], r["n_window"]) == (rin, rtot), t
        assert np.array_equal(r["num"], rnum), t
        if t == "DRs" and g.meta["drs_as_wgg"]:
            check_sums(r["sums"][..., :1], rsums[..., :1], label=t)
        else:
            check_sums(r["sums"], rsums, label=t)
    ctx.close()
