"""Parity at the full catalogue sizes of the two large workloads, on row
samples the oracle finishes in seconds: the 20,000,000-point clustered w++ box
(wgg + wg+ + w++, 125 jackknife cubes) and the sky survey with 500,000 data
points and 5,000,000 randoms (wg+, 100 regions, all four terms).  The GPU
counts the same outer rows of the full catalogues as the oracle; counts must be
identical and every field -- the cancelling shape sums included -- within 1e-6
relative per bin (and per Pi-integrated r_p profile) where the bin holds at
least 1% of the field's largest value, 1e-6 of that value elsewhere."""
import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import check_sums

pytestmark = pytest.mark.gpu


def _check(r, num, sums, n_total, n_in, label):
    assert (r["n_binned"], r["n_window"]) == (n_in, n_total), label
    assert np.array_equal(r["num"], num), label
    check_sums(r["sums"], sums, label=label)


def test_box_20M_wpp_row_sample_matches_oracle():
    wl = synth.box_ns_large_wpp()
    p = wl.params
    assert wl.shape.n > 19_900_000
    cats = host.prepare(p, [("S", wl.shape), ("D", wl.density)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    ocats = oracle.read_like_reference(p, [("S", wl.shape), ("D", wl.density)])
    stride = 200_000  # about 100 outer rows, ~1.3e7 binned pairs
    for offset in (0, 77_777):
        num, sums, n_total, n_in = oracle.port_corels2(p, "SD", ocats["D"], ocats["S"],
                                                       row_stride=stride, row_offset=offset)
        r = ctx.count("SD", 0, 1, row_stride=stride, row_offset=offset)
        _check(r, num, sums, n_total, n_in, f"20M box rows {offset} mod {stride}")
    ctx.close()


def test_box_2M_wpp_twin_count_equals_every_order_count():
    """The 2M-point clustered w++ box (the 20M box's geometry at a tenth of the
    points) in full: the twin count (each unordered pair tested once, both
    orders added) equals the count of every order -- counts identical, every
    field within the bar -- and so do its window pairs."""
    wl = synth.box_ns_large_wpp(n_parents=20000)
    p = wl.params
    cats = host.prepare(p, [("S", wl.shape), ("D", wl.density)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    rt = ctx.count("SD", 0, 1)
    assert ctx.last_twin()
    ctx.set_twin(False)
    ro = ctx.count("SD", 0, 1)
    assert not ctx.last_twin()
    assert (rt["n_binned"], rt["n_window"]) == (ro["n_binned"], ro["n_window"])
    assert np.array_equal(rt["num"], ro["num"])
    check_sums(rt["sums"], ro["sums"], label="twin vs every order")
    ctx.close()


def test_sky_500k_5M_row_sample_matches_oracle():
    wl = synth.sky_wgp(500_000, 5_000_000)
    p = wl.params
    order = [("S", wl.shape), ("Rs", wl.shape_rand), ("D", wl.density), ("Rd", wl.density_rand)]
    cats = host.prepare(p, order, table=wl.table)
    slots = {"S": 0, "Rs": 1, "D": 2, "Rd": 3}
    ctx = _lib.Context(p, table=wl.table)
    for role, slot in slots.items():
        ctx.upload(slot, cats[role])
    ocats = oracle.read_like_reference(p, order, table=wl.table)
    zsep = synth.derived_z_sep(p, wl.table)[0]
    terms = (("SRd", "Rd", "S"), ("RsRd", "Rd", "Rs"), ("SD", "D", "S"), ("DRs", "Rs", "D"))
    for kind, a, b in terms:
        n1 = max(cats[a].n, cats[b].n)
        stride = max(1, n1 // 150)  # about 150 outer rows of the larger catalogue
        num, sums, n_total, n_in = oracle.port_corels2(p, kind, ocats[a], ocats[b],
                                                       row_stride=stride, row_offset=11,
                                                       H_z=wl.table.H,
                                                       dA_z=wl.table.transverse, z_sep_max=zsep)
        r = ctx.count(kind, slots[a], slots[b], row_stride=stride, row_offset=11)
        _check(r, num, sums, n_total, n_in, f"sky {kind}")
    ctx.close()
