"""Auto pairs (corels1, estimators 1-3) on the GPU against the reference's own
auto-correlation runs and the oracle: every pair of one catalogue once by input
order, the sorted scan's +1 z image from row 0, images whose first scanned row
fails the redshift bound dropped."""
import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import AutoGolden, auto_golden_names, check_sums

pytestmark = pytest.mark.gpu


def _run_terms(g, engine):
    p = g.params
    cats = host.prepare(p, g.read_order(), table=g.table)
    ctx = _lib.Context(p, table=g.table)
    slots = {"S": 0, "Rs": 1}
    for r in g.cats:
        ctx.upload(slots[r], cats[r])
    out = {}
    for t in g.terms:
        if t == "SS":
            out[t] = ctx.count_auto("SS", 0, engine=engine)
        elif t == "RsRs":
            out[t] = ctx.count_auto("RsRs", 1, engine=engine)
        elif t == "SRs":
            out[t] = ctx.count("SRs", 1, 0, engine=engine)
    ctx.close()
    return out


@pytest.mark.parametrize("engine", ["fast", "fp64"])
@pytest.mark.parametrize("name", auto_golden_names())
def test_auto_matches_reference(name, engine):
    g = AutoGolden(name)
    got = _run_terms(g, engine)
    for t, r in got.items():
        rnum, rsums, rin, rtot = g.term(t)
        assert (r["n_binned"], r["n_window"]) == (rin, rtot), t
        assert np.array_equal(r["num"], rnum), t
        check_sums(r["sums"], rsums, label=t)


def test_auto_clustered_box_matches_oracle():
    """A clustered periodic box, w++ estimator 1, 27 cubes: fast and FP64
    engines equal the oracle's corels1 (counts exact, sums within 1e-6)."""
    c = synth.neyman_scott(300, 80.0, 2.0, 300.0, 61, nside_jk=3)
    p = synth._box_params(which_corr=2, L=300.0, rmin=0.1, rmax=40.0, nrp=16, npi=24, pmax=60.0,
                          njk=27, n=c.n)
    p.estimator = 1
    cats = host.prepare(p, [("S", c)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["S"])
    fast = ctx.count_auto("SS", 0)
    fp64 = ctx.count_auto("SS", 0, engine="fp64")
    ocats = oracle.read_like_reference(p, [("S", c)])
    num, sums, n_total, n_in = oracle.port_corels1(p, "SS", ocats["S"])
    for r in (fast, fp64):
        assert (r["n_binned"], r["n_window"]) == (n_in, n_total)
        assert np.array_equal(r["num"], num)
        check_sums(r["sums"], sums)
    ctx.close()


def test_auto_rejects_bad_kind():
    g = AutoGolden(auto_golden_names()[0])
    cats = host.prepare(g.params, g.read_order(), table=g.table)
    ctx = _lib.Context(g.params, table=g.table)
    ctx.upload(0, cats["S"])
    with pytest.raises(_lib.CpcError):
        ctx.count_auto("SD", 0)
    with pytest.raises(_lib.CpcError):
        ctx.count("SS", 0, 0)
    ctx.close()
