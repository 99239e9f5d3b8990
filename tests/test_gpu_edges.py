"""Edge cases against the oracle: empty and one-row catalogues, duplicated
positions (pairs at r_p = 0, orientation atan(0/0) = NaN as in the reference),
the largest supported binning (64 r_p x 128 Pi bins)."""
import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import check_sums

pytestmark = pytest.mark.gpu


def _cat(x, y, z, **kw):
    return synth.Catalog(np.asarray(x, float), np.asarray(y, float), np.asarray(z, float),
                         kw.get("w"), kw.get("e1"), kw.get("e2"), kw.get("jk"))


def _oracle_sd(p, S, D):
    o = oracle.read_like_reference(p, [("S", S), ("D", D)])
    return oracle.port_corels2(p, "SD", o["D"], o["S"])


def _gpu_sd(p, S, D, engine="fast"):
    cats = host.prepare(p, [("S", S), ("D", D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    r = ctx.count("SD", 0, 1, engine=engine)
    ctx.close()
    return r


def _assert_same(r, ref, nan_ok=False):
    num, sums, n_total, n_in = ref
    assert (r["n_binned"], r["n_window"]) == (n_in, n_total)
    assert np.array_equal(r["num"], num)
    if nan_ok:
        assert np.array_equal(np.isnan(r["sums"]), np.isnan(sums))
        g = np.where(np.isnan(sums), 0.0, r["sums"])
        s = np.where(np.isnan(sums), 0.0, sums)
        check_sums(g, s)
    else:
        check_sums(r["sums"], sums)


@pytest.mark.parametrize("engine", ["fast", "fp64"])
def test_empty_catalogues(engine):
    p = synth._box_params(which_corr=1, L=50.0, rmin=0.5, rmax=10.0, nrp=6, npi=8, pmax=20.0,
                          njk=0, n=0)
    full = synth.uniform_box(300, 50.0, 3, with_shapes=True)
    empty = _cat([], [], [])
    for S, D in ((empty, full), (full, empty), (empty, empty)):
        p.n_shape, p.n_density = S.n, D.n
        r = _gpu_sd(p, S, D, engine)
        assert r["n_binned"] == 0 and r["n_window"] == 0 and r["num"].sum() == 0
        assert not r["sums"].any()
    p.estimator = 1
    cats = host.prepare(p, [("S", empty)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["S"])
    r = ctx.count_auto("SS", 0, engine=engine)
    assert r["n_binned"] == 0 and r["num"].sum() == 0
    ctx.close()


@pytest.mark.parametrize("engine", ["fast", "fp64"])
def test_one_row_catalogue(engine):
    """A single galaxy paired with itself: one window pair (r_p = 0, Pi = 0),
    outside the log bins; and with linear bins from 0 it lands in bin 0."""
    for lin in (0, 1):
        p = synth._box_params(which_corr=0, L=50.0, rmin=0.0 if lin else 0.5, rmax=10.0, nrp=5,
                              npi=4, pmax=10.0, njk=0, n=1)
        p.lin_bin = lin
        c = _cat([25.0], [25.0], [25.0])
        _assert_same(_gpu_sd(p, c, c, engine), _oracle_sd(p, c, c))


@pytest.mark.parametrize("engine", ["fast", "fp64"])
def test_duplicated_positions(engine):
    """Every galaxy twice, linear r_p bins from 0 and shapes: the coincident
    pairs bin at r_p = 0 with the reference's NaN orientation."""
    base = synth.uniform_box(400, 60.0, 7, with_shapes=True, nside_jk=2)
    c = synth.Catalog(np.repeat(base.x, 2), np.repeat(base.y, 2), np.repeat(base.z, 2), None,
                      np.repeat(base.e1, 2), np.repeat(base.e2, 2), np.repeat(base.jk, 2))
    p = synth._box_params(which_corr=1, L=60.0, rmin=0.0, rmax=12.0, nrp=6, npi=6, pmax=15.0,
                          njk=8, n=c.n)
    p.lin_bin = 1
    _assert_same(_gpu_sd(p, c, c, engine), _oracle_sd(p, c, c), nan_ok=True)


@pytest.mark.parametrize("engine", ["fast", "fp64"])
def test_largest_binning(engine):
    c = synth.uniform_box(3000, 80.0, 9, with_shapes=True, nside_jk=2)
    p = synth._box_params(which_corr=2, L=80.0, rmin=0.05, rmax=30.0, nrp=64, npi=128,
                          pmax=40.0, njk=8, n=c.n)
    _assert_same(_gpu_sd(p, c, c, engine), _oracle_sd(p, c, c))
