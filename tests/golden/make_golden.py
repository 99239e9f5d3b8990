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
              "bins_cross_jk_final.dat", "bins2D_cross_jk_final.dat", "inp2.info"]


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
        for a in ("w", "e1", "e2", "jk"):
            v = getattr(c, a)
            if v is not None:
                arrays[f"{role}_{a}"] = v
    meta = {"name": name, "params": params, "same_files": same,
            "files": files}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print(f"{name}: n_in={sd['n_in']} n_total={totals[-1][0]} files={len(files)}")


def main():
    oracle.build_reference()
    for name, p, S, D, same in cases():
        run_case(name, p, S, D, same)


if __name__ == "__main__":
    main()
