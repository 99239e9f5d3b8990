"""The kappa, shape-kappa and ED accumulators (which_corr 3, 4, 5) and the r-mu
binning (coordinates 7) at sizes beyond the golden runs, against the oracle:
clustered boxes in full or on row samples, both engines, and the mu-slice
path that a binning too large for one block's shared memory takes."""
import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import check_sums

pytestmark = pytest.mark.gpu


def _run(p, S, D, *, engines=("fast", "fp64"), row_stride=1, row_offset=0):
    order = [("S", S), ("D", D)]
    ocats = oracle.read_like_reference(p, order)
    ref = oracle.port_corels2(p, "SD", ocats["D"], ocats["S"], row_stride=row_stride,
                              row_offset=row_offset)
    cats = host.prepare(p, order)
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    for eng in engines:
        r = ctx.count("SD", 0, 1, engine=eng, row_stride=row_stride, row_offset=row_offset)
        assert (r["n_binned"], r["n_window"]) == (ref[3], ref[2]), eng
        assert np.array_equal(r["num"], ref[0]), eng
        check_sums(r["sums"], ref[1], label=eng)
    ctx.close()


def test_ed_rmu_clustered():
    """The ED notebook's run shape (r-mu, one mu bin) and a finer mu binning."""
    c = synth.with_orientation(synth.neyman_scott(300, 60.0, 2.0, 75.0, 61, nside_jk=3), 62)
    for npi in (1, 8):
        p = synth._box_params(which_corr=5, L=75.0, rmin=0.1, rmax=10.0, nrp=10, npi=npi,
                              pmax=1.0, njk=27, n=c.n)
        p.coordinates = 7
        _run(p, c, c)


def test_kappa_density_clustered():
    """The size notebook's run shape (which_corr 3, r_p-Pi, unsorted)."""
    c = synth.neyman_scott(400, 60.0, 2.0, 75.0, 63, nside_jk=3)
    c = synth.with_kappa(c.subset(np.random.default_rng(64).permutation(c.n)), 65)
    p = synth._box_params(which_corr=3, L=75.0, rmin=0.1, rmax=10.0, nrp=10, npi=20, pmax=25.0,
                          njk=27, n=c.n)
    p.data_sorted = 0
    _run(p, c, c)


def test_shape_kappa_swap():
    """which_corr 4 with the larger catalogue second (the g1/g2 swap)."""
    s = synth.uniform_box(6000, 100.0, 66, nside_jk=2, with_shapes=True)
    d = synth.with_kappa(synth.uniform_box(15000, 100.0, 67, nside_jk=2), 68)
    p = synth._box_params(which_corr=4, L=100.0, rmin=0.3, rmax=15.0, nrp=8, npi=10,
                          pmax=20.0, njk=8, n=0)
    p.n_shape, p.n_density = s.n, d.n
    _run(p, s, d)


def test_rmu_mu_slices():
    """w++ in r-mu with 40 x 100 bins: the per-block histograms do not fit
    shared memory, so the units are repeated over slices of mu bins."""
    c = synth.neyman_scott(200, 50.0, 2.0, 100.0, 69, nside_jk=2)
    p = synth._box_params(which_corr=2, L=100.0, rmin=0.1, rmax=20.0, nrp=40, npi=100, pmax=1.0,
                          njk=8, n=c.n)
    p.coordinates = 7
    _run(p, c, c, engines=("fast", "cell_fp64"))


def test_ed_rppi_large_row_sample():
    """ED in r_p-Pi on the 200,000-galaxy clustered box, every 53rd outer row."""
    wl = synth.box_ns_wgp()
    c = synth.with_orientation(wl.shape, 70)
    p = wl.params
    p.which_corr = 5
    _run(p, c, c, row_stride=53, row_offset=3)


def test_variants_rejected_where_the_reference_has_no_box_computation():
    p = synth._sky_params(which_corr=5, rmin=0.3, rmax=30.0, nrp=8, npi=12, pmax=40.0, njk=0)
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    with pytest.raises(_lib.CpcError):
        _lib.Context(p, table=t)
    p = synth._box_params(which_corr=1, L=75.0, rmin=0.1, rmax=10.0, nrp=10, npi=4, pmax=1.0,
                          njk=0, n=0)
    p.coordinates = 7
    p.periodic_box = 0
    with pytest.raises(_lib.CpcError):
        _lib.Context(p)
