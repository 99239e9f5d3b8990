"""The benchmark's synthetic workloads match the configurations they stand in
for: sizes, value ranges and distributions, jackknife grids and bins (CPU only).

The configurations are the reference's benchmark list: a 20k uniform wgg box, the
200k Neyman-Scott wg+ box, the 500k + 5M sky survey, 64 uneven w++ sub-boxes and
the 20M Neyman-Scott w++ box."""
import inspect

import numpy as np
import pytest

from corr_pc_gb300 import synth


def _check_box_params(p, *, which_corr, L, rmin, rmax, nrp, npi, pmax, njk, n):
    assert p.which_corr == which_corr and p.coordinates == 6
    assert p.periodic_box == 1 and p.periodic_box_size == L
    assert (p.bin_r_min, p.bin_r_max, p.n_bins, p.lin_bin) == (rmin, rmax, nrp, 0)
    assert (p.n_p_bin, p.p_min, p.p_max) == (npi, -pmax, pmax)
    assert p.do_jk == 1 and p.n_jk_regions == njk
    assert p.n_shape == n and p.n_density == n
    assert p.data_sorted == 1


def _check_box_catalog(c, L, nside, *, float32, shapes_expected=True):
    for v in (c.x, c.y, c.z):
        assert v.dtype == np.float64
        assert v.min() >= 0.0 and v.max() < L
        if float32:
            assert np.array_equal(v.astype(np.float32).astype(np.float64), v)
    assert np.all(np.diff(c.z) >= 0)            # sorted by z (data_sorted 1)
    assert c.w is None                          # weights all 1
    assert c.jk is not None
    assert c.jk.min() >= 0 and c.jk.max() < nside ** 3
    assert np.array_equal(c.jk, synth.jk_cubes(c.x, c.y, c.z, L, nside))
    if shapes_expected:
        _check_shapes(c.e1, c.e2)


def _check_shapes(e1, e2):
    assert e1 is not None and e2 is not None
    assert np.all(e1 * e1 + e2 * e2 < 1.0)      # truncated to |e| < 1
    # N(0, 0.25) per component before truncation: |e|^2 ~ Exp(mean m = 0.5);
    # cut at 1 it has mean m - q/(1-q), q = exp(-1/m), half of it per component
    m = 0.5
    q = np.exp(-1.0 / m)
    sd = np.sqrt(0.5 * (m - q / (1.0 - q)))
    assert abs(sd - 0.4145) < 1e-3
    for e in (e1, e2):
        assert abs(e.mean()) < 0.01
        assert abs(e.std() - sd) < 0.01


def test_box_uniform_wgg_20k():
    wl = synth.box_uniform_wgg()
    assert wl.name == "box_uniform_wgg_20k" and wl.shape is wl.density
    c = wl.shape
    assert c.n == 20000
    _check_box_params(wl.params, which_corr=0, L=250.0, rmin=0.1, rmax=20.0, nrp=10,
                      npi=20, pmax=100.0, njk=8, n=20000)
    _check_box_catalog(c, 250.0, 2, float32=False, shapes_expected=False)
    assert np.bincount(c.jk, minlength=8).min() > 2000   # uniform over the 8 cubes
    # seed 0 gives the same catalogue every time
    c2 = synth.box_uniform_wgg().shape
    assert np.array_equal(c.x, c2.x) and np.array_equal(c.z, c2.z)


def test_box_ns_wgp_200k():
    wl = synth.box_ns_wgp()
    assert wl.name == "box_ns_wgp_200k"
    c = wl.shape
    # 2,000 parents x Poisson(100): 200,000 +- 5 sigma; seed 0 gives 199,865
    assert abs(c.n - 200000) < 5 * np.sqrt(200000)
    assert c.n == 199865
    _check_box_params(wl.params, which_corr=1, L=500.0, rmin=0.1, rmax=60.0, nrp=20,
                      npi=40, pmax=100.0, njk=64, n=c.n)
    _check_box_catalog(c, 500.0, 4, float32=True)
    assert np.bincount(c.jk, minlength=64).min() > 0


def test_neyman_scott_offsets():
    """Children sit at Gaussian offsets of the stated sigma from their parent
    (checked with one parent far from the walls)."""
    L, sigma = 1000.0, 2.0
    c = synth.neyman_scott(1, 5000.0, sigma, L, 7, float32=False, with_shapes=False)
    rng = np.random.default_rng(7)
    parent = rng.uniform(0.0, L, size=(1, 3))[0]
    assert np.all(parent > 50) and np.all(parent < L - 50)
    off = np.stack([c.x, c.y, c.z], axis=1) - parent
    assert abs(c.n - 5000) < 5 * np.sqrt(5000)
    assert np.all(np.abs(off.mean(axis=0)) < 0.1)
    assert np.all(np.abs(off.std(axis=0) - sigma) < 0.1)


def test_box_variants_200k():
    """The ED (r-mu) and kappa workloads are the same 200k box with one more
    per-galaxy column."""
    base = synth.box_ns_wgp().shape
    ed = synth.box_ns_ed_rmu()
    assert ed.params.which_corr == 5 and ed.params.coordinates == 7
    assert (ed.params.n_p_bin, ed.params.p_min, ed.params.p_max) == (10, -1.0, 1.0)
    assert np.array_equal(ed.shape.x, base.x) and ed.shape.e3 is not None
    kap = synth.box_ns_kappa()
    assert kap.params.which_corr == 3 and kap.shape.e2 is None
    assert np.array_equal(kap.shape.z, base.z)
    assert abs(kap.shape.e1.mean()) < 1e-12   # mean-subtracted


def test_box_batch_wpp_64():
    sizes = synth.box_batch_sizes()
    assert sizes.shape == (64,)
    assert sizes.min() >= 10000 and sizes.max() < 400000
    # log-uniform from 1e4 to 4e5
    u = (np.log(sizes) - np.log(1e4)) / (np.log(4e5) - np.log(1e4))
    assert 0.35 < u.mean() < 0.65
    assert np.array_equal(sizes, synth.box_batch_sizes())   # seeded
    wls = synth.box_batch_wpp(scale=0.01)
    assert len(wls) == 64
    for wl, nb in zip(wls, sizes):
        assert wl.shape.n == max(2, int(nb * 0.01))
        _check_box_params(wl.params, which_corr=2, L=200.0, rmin=0.1, rmax=60.0, nrp=20,
                          npi=40, pmax=100.0, njk=27, n=wl.shape.n)
    big = synth.box_batch_wpp(n_boxes=2, scale=0.2)
    for wl in big:
        _check_box_catalog(wl.shape, 200.0, 3, float32=False)
    sig = inspect.signature(synth.box_batch_wpp).parameters
    assert sig["n_boxes"].default == 64 and sig["scale"].default == 1.0


def test_box_ns_wpp_20M_parameters():
    """The 20M box's parameters, on a catalogue with 1/100 of its parents (the
    full catalogue takes several GB of host memory to make)."""
    sig = inspect.signature(synth.box_ns_large_wpp).parameters
    assert sig["n_parents"].default == 200000
    wl = synth.box_ns_large_wpp(n_parents=2000)
    assert wl.name == "box_ns_wpp_20M"
    c = wl.shape
    assert abs(c.n - 200000) < 5 * np.sqrt(200000)
    _check_box_params(wl.params, which_corr=2, L=1000.0, rmin=0.1, rmax=100.0, nrp=25,
                      npi=50, pmax=100.0, njk=125, n=c.n)
    _check_box_catalog(c, 1000.0, 5, float32=True)


def test_sky_wgp_500k_5M_parameters():
    """The sky survey's parameters and distributions, on 40k data and 100k
    randoms (the generator's defaults are the full 500k and 5M)."""
    sig = inspect.signature(synth.sky_wgp).parameters
    assert sig["n_data"].default == 500000 and sig["n_rand"].default == 5000000
    wl = synth.sky_wgp(40000, 100000)
    p = wl.params
    assert p.coordinates == 0 and p.periodic_box == 0 and p.use_comoving == 1
    assert (p.bin_r_min, p.bin_r_max, p.n_bins, p.lin_bin) == (0.3, 60.0, 15, 0)
    assert (p.n_p_bin, p.p_min, p.p_max) == (30, -60.0, 60.0)
    assert p.do_jk == 1 and p.n_jk_regions == 100
    assert wl.shape is wl.density and wl.shape_rand is wl.density_rand
    d, r = wl.shape, wl.shape_rand
    assert d.n == 40000 and r.n == 100000
    _check_shapes(d.e1, d.e2)
    assert d.w.min() >= 0.5 and d.w.max() < 1.5 and abs(d.w.mean() - 1.0) < 0.01
    assert r.w is None and r.e1 is None
    for c in (d, r):
        ra, dec = c.x, c.y
        assert ra.min() >= 0.0 and ra.max() < 10.0
        assert dec.min() >= 0.0 and dec.max() < 10.0
        # uniform on the sphere: sin(Dec) uniform on [0, sin 10 deg)
        s = np.sin(np.radians(dec)) / np.sin(np.radians(10.0))
        assert abs(s.mean() - 0.5) < 0.01
        assert np.all(np.diff(c.z) >= 0)
        chi = np.interp(c.z, wl.table.z, wl.table.DC)
        assert chi.min() > 499.9 and chi.max() < 1500.1
        # n(chi) ~ chi^2: chi^3 uniform on [500^3, 1500^3]
        u = (chi ** 3 - 500.0 ** 3) / (1500.0 ** 3 - 500.0 ** 3)
        assert abs(u.mean() - 0.5) < 0.01
        assert c.jk.min() >= 0 and c.jk.max() < 100
        assert np.bincount(c.jk, minlength=100).min() > 0
        assert np.array_equal(c.jk, synth.jk_sky_grid(ra, dec, (0, 10), (0, 10), 10, 10))
    # the distance table covers the redshifts the patch needs
    assert wl.table.z[-1] >= p.z_max and d.z.max() < p.z_max


@pytest.mark.parametrize("nside", [2, 3, 4, 5])
def test_jk_cubes_labels(nside):
    L = 100.0
    g = (np.arange(nside) + 0.5) * L / nside
    x, y, z = (a.ravel() for a in np.meshgrid(g, g, g, indexing="ij"))
    lab = synth.jk_cubes(x, y, z, L, nside)
    assert sorted(lab.tolist()) == list(range(nside ** 3))
    edge = synth.jk_cubes(np.array([np.nextafter(L, 0)]), np.zeros(1), np.zeros(1), L, nside)
    assert edge[0] == (nside - 1) * nside * nside
