"""Generate the golden fixtures by running the REFERENCE corr_pc itself.

Each case is a small seeded catalogue pair written in the reference's input
format with a positional .inp; the reference harness (oracle/ref_harness.cpp,
built by oracle/Makefile from the reference's own sources) replays do_corr,
dumps every raw histogram tree and writes the reference's output files.  The
fixture stores the inputs, the raw sums (region sums recovered from the
delete-one samples), the pair counters and a selection of the output files.

Run where the reference sources are available:
    python tests/golden/make_golden.py
The fixtures (tests/golden/*.npz) are committed; tests only read them.
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from corr_pc_gb300 import synth  # noqa: E402

KEEP_FILES = ["bins_cross_final.dat", "bins2D_cross_final.dat", "bins_cross_SD.dat",
              "bins2D_cross_SD.dat", "bins_cross_RR.dat", "bins2D_cross_RR.dat",
              "bins_cross_SR.dat", "bins_cross_jk0_final.dat", "bins2D_cross_jk0_SD.dat",
              "bins_cross_jk_final.dat", "bins2D_cross_jk_final.dat", "inp2.info",
              "bins_auto_final.dat", "bins2D_auto_final.dat", "bins_auto_SS.dat",
              "bins2D_auto_SS.dat", "bins_auto_RR.dat", "bins2D_auto_RR.dat", "bins_auto_SR.dat",
              "bins_auto_jk0_final.dat", "bins2D_auto_jk0_SS.dat", "bins_auto_jk_final.dat",
              "bins2D_auto_jk_final.dat"]


def lattice(n, L, seed, jk_side):
    """Integer lattice points: separations land exactly on bin edges."""
    rng = np.random.default_rng(seed)
    xyz = rng.integers(0, int(L), size=(3, n)).astype(np.float64)
    x, y, z = xyz
    jk = synth.jk_cubes(x, y, z, L, jk_side)
    return synth.Catalog(x, y, z, None, None, None, jk).sorted_by_z()


def cases():
    out = []
    c = synth.uniform_box(3000, 100.0, 11, nside_jk=2)
    p = synth._box_params(which_corr=0, L=100.0, rmin=0.5, rmax=20.0, nrp=8, npi=12, pmax=30.0,
                          njk=8, n=c.n)
    out.append(("box_wgg_uniform", p, c, c, True))

    c = synth.neyman_scott(40, 50.0, 2.0, 120.0, 12, nside_jk=3)
    p = synth._box_params(which_corr=1, L=120.0, rmin=0.1, rmax=30.0, nrp=12, npi=16, pmax=40.0,
                          njk=27, n=c.n)
    out.append(("box_wgp_clustered", p, c, c, True))

    c = synth.uniform_box(2500, 100.0, 13, nside_jk=2, with_shapes=True)
    p = synth._box_params(which_corr=2, L=100.0, rmin=0.2, rmax=25.0, nrp=10, npi=10, pmax=30.0,
                          njk=8, n=c.n)
    out.append(("box_wpp_uniform", p, c, c, True))

    rng = np.random.default_rng(14)
    s = synth.uniform_box(1500, 80.0, 15, nside_jk=2, with_shapes=True)
    d = synth.uniform_box(2200, 80.0, 16, nside_jk=2, with_shapes=True)
    s.w = rng.uniform(0.5, 1.5, s.n)
    d.w = rng.uniform(0.5, 1.5, d.n)
    p = synth._box_params(which_corr=2, L=80.0, rmin=0.5, rmax=20.0, nrp=8, npi=10, pmax=25.0,
                          njk=8, n=0)
    p.n_shape, p.n_density = s.n, d.n
    out.append(("box_wpp_weighted_distinct", p, s, d, False))

    s = synth.uniform_box(3000, 90.0, 17, nside_jk=2, with_shapes=True)
    d = synth.uniform_box(1200, 90.0, 18, nside_jk=2, with_shapes=True)
    p = synth._box_params(which_corr=1, L=90.0, rmin=0.3, rmax=20.0, nrp=8, npi=10, pmax=30.0,
                          njk=8, n=0)
    p.n_shape, p.n_density = s.n, d.n
    out.append(("box_wgp_swap", p, s, d, False))

    c = synth.uniform_box(2000, 60.0, 19)
    p = synth._box_params(which_corr=0, L=60.0, rmin=0.0, rmax=20.0, nrp=10, npi=8, pmax=20.0,
                          njk=0, n=c.n)
    p.lin_bin = 1
    out.append(("box_linear_bins_nojk", p, c, c, True))

    c = lattice(700, 40.0, 20, 2)
    p = synth._box_params(which_corr=0, L=40.0, rmin=1.0, rmax=16.0, nrp=4, npi=8, pmax=8.0,
                          njk=8, n=c.n)
    out.append(("box_lattice_edges", p, c, c, True))

    c = synth.neyman_scott(30, 60.0, 2.0, 100.0, 21, nside_jk=2)
    perm = np.random.default_rng(22).permutation(c.n)
    c = c.subset(perm)
    p = synth._box_params(which_corr=1, L=100.0, rmin=0.2, rmax=25.0, nrp=10, npi=10, pmax=30.0,
                          njk=8, n=c.n)
    p.data_sorted = 0
    out.append(("box_wgp_unsorted", p, c, c, True))

    # the variants: kappa-density (which_corr 3), shape-kappa (4), ED (5), and
    # r-mu binning (coordinates 7) -- the ED and size notebooks' settings
    c = synth.with_orientation(synth.neyman_scott(30, 40.0, 2.0, 75.0, 31, nside_jk=2), 32)
    p = synth._box_params(which_corr=5, L=75.0, rmin=0.1, rmax=10.0, nrp=10, npi=4, pmax=1.0,
                          njk=8, n=c.n)
    p.coordinates = 7
    out.append(("box_ed_rmu", p, c, c, True))

    c = synth.with_orientation(synth.uniform_box(2500, 80.0, 33, nside_jk=2), 34)
    p = synth._box_params(which_corr=5, L=80.0, rmin=0.3, rmax=15.0, nrp=8, npi=10, pmax=20.0,
                          njk=8, n=c.n)
    out.append(("box_ed_rppi", p, c, c, True))

    c = synth.neyman_scott(30, 50.0, 2.0, 75.0, 35, nside_jk=3)
    c = synth.with_kappa(c.subset(np.random.default_rng(36).permutation(c.n)), 37)
    p = synth._box_params(which_corr=3, L=75.0, rmin=0.1, rmax=10.0, nrp=10, npi=20, pmax=25.0,
                          njk=27, n=c.n)
    p.data_sorted = 0
    out.append(("box_kappa_unsorted", p, c, c, True))

    rng = np.random.default_rng(38)
    s = synth.uniform_box(1800, 80.0, 39, nside_jk=2, with_shapes=True)
    d = synth.with_kappa(synth.uniform_box(2400, 80.0, 40, nside_jk=2), 41)
    s.w = rng.uniform(0.5, 1.5, s.n)
    p = synth._box_params(which_corr=4, L=80.0, rmin=0.3, rmax=15.0, nrp=8, npi=10, pmax=20.0,
                          njk=8, n=0)
    p.n_shape, p.n_density = s.n, d.n
    out.append(("box_sk_distinct", p, s, d, False))

    c = synth.uniform_box(2500, 90.0, 42, nside_jk=2, with_shapes=True)
    p = synth._box_params(which_corr=2, L=90.0, rmin=0.0, rmax=18.0, nrp=9, npi=10, pmax=1.0,
                          njk=8, n=c.n)
    p.coordinates = 7
    p.lin_bin = 1
    out.append(("box_wpp_rmu_linear", p, c, c, True))

    # integer lattice in r-mu: mu = 0 (Pi = 0) sits on a bin edge and mu = +-1
    # (dx = dy = 0) on the range ends; linear r bins put integer r on edges
    c = lattice(700, 40.0, 43, 2)
    p = synth._box_params(which_corr=0, L=40.0, rmin=0.0, rmax=12.0, nrp=6, npi=4, pmax=1.0,
                          njk=8, n=c.n)
    p.coordinates = 7
    p.lin_bin = 1
    out.append(("box_lattice_rmu", p, c, c, True))
    return out


def run_case(name, p, S, D, same):
    with tempfile.TemporaryDirectory() as tmp:
        wl = synth.Workload(name, p, S, D)
        inp = synth.write_box_run(tmp, wl, same_files=same, n_threads=1)
        totals, _ = oracle.run_reference(inp, os.path.join(tmp, "dump.txt"), bining=True)
        dump = oracle.parse_dump(os.path.join(tmp, "dump.txt"))
        files = {}
        for f in KEEP_FILES:
            fp = os.path.join(tmp, "out", "run_" + f)
            if os.path.exists(fp):
                files[f] = open(fp).read()
        params = {a: getattr(p, a) for _k, a, _t in synth.INP_KEYS}
    sd = dump["SD"]
    arrays = {
        "S_x": S.x, "S_y": S.y, "S_z": S.z, "D_x": D.x, "D_y": D.y, "D_z": D.z,
        "raw_num": sd["raw_num"], "raw_sums": sd["raw_sums"],
        "n_in": np.array(sd["n_in"]), "n_total": np.array(totals[-1][0]),
    }
    for role, c in (("S", S), ("D", D)):
        for a in ("w", "e1", "e2", "e3", "jk"):
            v = getattr(c, a)
            if v is not None:
                arrays[f"{role}_{a}"] = v
    meta = {"name": name, "params": params, "same_files": same,
            "files": files}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print(f"{name}: n_in={sd['n_in']} n_total={totals[-1][0]} files={len(files)}")


SKY_TERMS = ("SRd", "RsRd", "SD", "DRs")  # do_corr.cpp:98-133 order


def sky_cases():
    """Sky cross runs (coordinates 0): data and randoms on a small RA/Dec patch
    with a flat LCDM distance table on a coarse dz grid (keeps the fixture
    small; the table is stored in the fixture)."""
    out = []
    p = synth._sky_params(which_corr=1, rmin=0.3, rmax=30.0, nrp=8, npi=12, pmax=40.0,
                          njk=9, z_max=0.5)
    p.dz = 0.001
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    d = synth.sky_patch(1500, 31, t, ra_deg=6, dec_deg=6, chi_range=(500, 900), nside_jk=3,
                        with_shapes=True, weights=True)
    r = synth.sky_patch(4000, 32, t, ra_deg=6, dec_deg=6, chi_range=(500, 900), nside_jk=3)
    out.append(("sky_wgp_jk", synth.SkyWorkload("sky_wgp_jk", p, t, d, d, r, r), True))

    p = synth._sky_params(which_corr=0, rmin=0.5, rmax=40.0, nrp=10, npi=10, pmax=50.0,
                          njk=4, z_max=0.6)
    p.dz = 0.001
    p.data_sorted = 0
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    # RA across 0/360 exercises the reference's RA wrap (sky_calcs.cpp:134-141)
    s = synth.sky_patch(1200, 33, t, ra_deg=8, dec_deg=30, chi_range=(600, 1200), nside_jk=2,
                        weights=True)
    dd = synth.sky_patch(900, 34, t, ra_deg=8, dec_deg=30, chi_range=(600, 1200), nside_jk=2)
    rs = synth.sky_patch(3000, 35, t, ra_deg=8, dec_deg=30, chi_range=(600, 1200), nside_jk=2)
    rd = synth.sky_patch(2500, 36, t, ra_deg=8, dec_deg=30, chi_range=(600, 1200), nside_jk=2)
    for c in (s, dd, rs, rd):
        c.x = np.where(c.x < 3.0, c.x + 357.0, c.x - 3.0)
        c.y = c.y - 10.0
    rng = np.random.default_rng(37)
    for c in (s, dd, rs, rd):  # unsorted input (data_sorted 0)
        perm = rng.permutation(c.n)
        c2 = c.subset(perm)
        c.x, c.y, c.z, c.w, c.e1, c.e2, c.jk = c2.x, c2.y, c2.z, c2.w, c2.e1, c2.e2, c2.jk
    out.append(("sky_wgg_distinct_wrap", synth.SkyWorkload("sky_wgg_distinct_wrap", p, t, s, dd,
                                                           rs, rd), False))

    # twins at almost exactly the clamp angle of dA_calc (sum = 0.9999999999,
    # theta ~ 1.41421e-5 rad): the pairs whose count depends on the last bits of
    # cos and acos, binned by the host edge tier
    p = synth._sky_params(which_corr=0, rmin=0.005, rmax=30.0, nrp=12, npi=8, pmax=40.0,
                          njk=4, z_max=0.5)
    p.dz = 0.001
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    base = synth.sky_patch(700, 38, t, ra_deg=4, dec_deg=4, chi_range=(600, 900), nside_jk=2)
    rng = np.random.default_rng(39)
    th = np.sqrt(2e-10) * (1.0 + rng.uniform(-3e-5, 3e-5, base.n))
    ang = rng.uniform(0, 2 * np.pi, base.n)
    th_deg = np.degrees(th)
    tw = synth.Catalog(base.x + th_deg * np.cos(ang) / np.cos(np.radians(base.y)),
                       base.y + th_deg * np.sin(ang), base.z.copy(), None, None, None,
                       base.jk.copy())
    both = synth.Catalog(np.concatenate([base.x, tw.x]), np.concatenate([base.y, tw.y]),
                         np.concatenate([base.z, tw.z]), None, None, None,
                         np.concatenate([base.jk, tw.jk])).sorted_by_z()
    r = synth.sky_patch(1500, 40, t, ra_deg=4, dec_deg=4, chi_range=(600, 900), nside_jk=2)
    out.append(("sky_twins_clamp", synth.SkyWorkload("sky_twins_clamp", p, t, both, both, r, r),
                True))

    # a box without periodic images (coordinates 6, periodic_box 0: lim_calc_xyz,
    # Landy-Szalay with randoms); the distances file is read but unused.  No
    # jackknife: lim_calc_xyz never sets the row's region (ct.gjk[0]) and the
    # reference crashes in corel_jk1 with do_jk on.
    p = _nbox_params(which_corr=1, njk=0)
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    d = _nbox_clustered(57)
    r = synth.uniform_box(3000, 100.0, 58, nside_jk=2)
    out.append(("nbox_wgp_ls", synth.SkyWorkload("nbox_wgp_ls", p, t, d, d, r, r), True))
    return out


def _nbox_params(*, which_corr, njk):
    p = synth._box_params(which_corr=which_corr, L=100.0, rmin=0.3, rmax=20.0, nrp=8, npi=10,
                          pmax=25.0, njk=njk, n=0)
    p.periodic_box = 0
    p.dz = 1.0
    p.z_max = 100.0
    return p


def _nbox_clustered(seed):
    """Neyman-Scott points inside [0, 100)^3 without wrapping (parents kept
    away from the faces)."""
    rng = np.random.default_rng(seed)
    parents = rng.uniform(10.0, 90.0, size=(40, 3))
    counts = rng.poisson(40, 40)
    pos = np.repeat(parents, counts, axis=0) + rng.normal(0.0, 2.0, size=(int(counts.sum()), 3))
    pos = np.clip(pos, 0.0, 99.999)
    e1, e2 = synth.shapes(rng, pos.shape[0])
    jk = synth.jk_cubes(pos[:, 0], pos[:, 1], pos[:, 2], 100.0, 2)
    return synth.Catalog(pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy(), None, e1, e2,
                         jk).sorted_by_z()


def run_sky_case(name, wl, same):
    with tempfile.TemporaryDirectory() as tmp:
        inp = synth.write_sky_run(tmp, wl, n_threads=1, same_files=same)
        totals, _ = oracle.run_reference(inp, os.path.join(tmp, "dump.txt"), bining=True,
                                         drs_wgg=True)
        dump = oracle.parse_dump(os.path.join(tmp, "dump.txt"))
        files = {}
        for f in KEEP_FILES:
            fp = os.path.join(tmp, "out", "run_" + f)
            if os.path.exists(fp):
                files[f] = open(fp).read()
        params = {a: getattr(wl.params, a) for _k, a, _t in synth.INP_KEYS}
    arrays = {"table_H": wl.table.H, "table_DC": wl.table.DC, "table_DA": wl.table.DA}
    for role, c in (("S", wl.shape), ("D", wl.density), ("Rs", wl.shape_rand),
                    ("Rd", wl.density_rand)):
        for a in ("x", "y", "z", "w", "e1", "e2", "jk"):
            v = getattr(c, a)
            if v is not None:
                arrays[f"{role}_{a}"] = v
    for k, term in enumerate(SKY_TERMS):
        arrays[f"{term}_raw_num"] = dump[term]["raw_num"]
        arrays[f"{term}_raw_sums"] = dump[term]["raw_sums"]
        arrays[f"{term}_n_in"] = np.array(dump[term]["n_in"])
        arrays[f"{term}_n_total"] = np.array(totals[k][0])
    meta = {"name": name, "params": params, "same_files": same, "files": files,
            "terms": list(SKY_TERMS), "drs_as_wgg": True}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print(f"{name}: " + " ".join(f"{t}={dump[t]['n_in']}" for t in SKY_TERMS))


def auto_cases():
    """Auto-correlation runs (estimator 1: corels1 on S; estimator 2 adds the
    Pi re-binning).  A periodic box counts SS only; the sky adds SRs and RsRs."""
    out = []
    c = synth.uniform_box(2500, 100.0, 51, nside_jk=2)
    p = synth._box_params(which_corr=0, L=100.0, rmin=0.5, rmax=20.0, nrp=8, npi=12, pmax=30.0,
                          njk=8, n=c.n)
    p.estimator = 1
    out.append(("auto_box_wgg", p, c, None, None))

    c = synth.uniform_box(2000, 100.0, 52, nside_jk=2, with_shapes=True)
    p = synth._box_params(which_corr=2, L=100.0, rmin=0.3, rmax=25.0, nrp=10, npi=10, pmax=30.0,
                          njk=8, n=c.n)
    p.estimator = 2
    out.append(("auto_box_wpp_rebin", p, c, None, None))

    c = synth.neyman_scott(30, 60.0, 2.0, 100.0, 53, nside_jk=2)
    c = c.subset(np.random.default_rng(54).permutation(c.n))
    p = synth._box_params(which_corr=1, L=100.0, rmin=0.2, rmax=25.0, nrp=10, npi=10, pmax=30.0,
                          njk=8, n=c.n)
    p.estimator = 1
    p.data_sorted = 0
    out.append(("auto_box_wgp_unsorted", p, c, None, None))

    # ED auto-correlation in r-mu (corels1 with ED_corel, g_with_shape 1)
    c = synth.with_orientation(synth.neyman_scott(25, 50.0, 2.0, 60.0, 57, nside_jk=2), 58)
    p = synth._box_params(which_corr=5, L=60.0, rmin=0.2, rmax=12.0, nrp=8, npi=6, pmax=1.0,
                          njk=8, n=c.n)
    p.coordinates = 7
    p.estimator = 1
    out.append(("auto_box_ed_rmu", p, c, None, None))

    p = synth._sky_params(which_corr=1, rmin=0.3, rmax=30.0, nrp=8, npi=12, pmax=40.0, njk=9,
                          z_max=0.5)
    p.dz = 0.001
    p.estimator = 1
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    d = synth.sky_patch(1500, 55, t, ra_deg=6, dec_deg=6, chi_range=(500, 900), nside_jk=3,
                        with_shapes=True, weights=True)
    r = synth.sky_patch(4000, 56, t, ra_deg=6, dec_deg=6, chi_range=(500, 900), nside_jk=3)
    out.append(("auto_sky_wgp", p, d, r, t))

    p = _nbox_params(which_corr=0, njk=0)
    p.estimator = 1
    t = synth.flat_lcdm_table(p.z_max, p.dz)
    out.append(("auto_nbox_wgg", p, _nbox_clustered(59),
                synth.uniform_box(2500, 100.0, 60, nside_jk=2), t))
    return out


def run_auto_case(name, p, S, R, table):
    with tempfile.TemporaryDirectory() as tmp:
        if table is None:
            inp = synth.write_box_run(tmp, synth.Workload(name, p, S, S), same_files=True,
                                      n_threads=1)
        else:
            inp = synth.write_sky_run(tmp, synth.SkyWorkload(name, p, table, S, S, R, R),
                                      n_threads=1)
        totals, _ = oracle.run_reference(inp, os.path.join(tmp, "dump.txt"), bining=True)
        dump = oracle.parse_dump(os.path.join(tmp, "dump.txt"))
        files = {}
        for f in KEEP_FILES:
            fp = os.path.join(tmp, "out", "run_" + f)
            if os.path.exists(fp):
                files[f] = open(fp).read()
        params = {a: getattr(p, a) for _k, a, _t in synth.INP_KEYS}
    terms = list(dump.keys())
    arrays = {}
    if table is not None:
        arrays.update({"table_H": table.H, "table_DC": table.DC, "table_DA": table.DA})
    for role, c in (("S", S), ("Rs", R)):
        if c is None:
            continue
        for a in ("x", "y", "z", "w", "e1", "e2", "e3", "jk"):
            v = getattr(c, a)
            if v is not None:
                arrays[f"{role}_{a}"] = v
    for k, term in enumerate(terms):
        arrays[f"{term}_raw_num"] = dump[term]["raw_num"]
        arrays[f"{term}_raw_sums"] = dump[term]["raw_sums"]
        arrays[f"{term}_n_in"] = np.array(dump[term]["n_in"])
        arrays[f"{term}_n_total"] = np.array(totals[k][0])
    meta = {"name": name, "params": params, "files": files, "terms": terms}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print(f"{name}: " + " ".join(f"{t}={dump[t]['n_in']}" for t in terms))


def main():
    oracle.build_reference()
    only = sys.argv[1:]
    for name, p, S, D, same in cases():
        if not only or name in only:
            run_case(name, p, S, D, same)
    for name, wl, same in sky_cases():
        if not only or name in only:
            run_sky_case(name, wl, same)
    for name, p, S, R, table in auto_cases():
        if not only or name in only:
            run_auto_case(name, p, S, R, table)


if __name__ == "__main__":
    main()
