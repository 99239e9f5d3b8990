"""The corr_pc_gb300 command line (the reference's argv, .inp and files) on
the golden cases: every output file equals the reference's."""
import json
import os
import subprocess

import pytest

from corr_pc_gb300 import build, synth
from helpers import Golden, compare_files

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["box_wgg_uniform", "box_wgp_clustered", "box_wpp_weighted_distinct",
                                  "box_wgp_swap", "box_linear_bins_nojk", "box_ed_rmu",
                                  "box_kappa_unsorted", "box_sk_distinct", "box_wpp_rmu_linear"])
def test_cli_output_files_match_reference(name, tmp_path):
    g = Golden(name)
    wl = synth.Workload(name, g.params, g.S, g.D)
    inp = synth.write_box_run(str(tmp_path), wl, same_files=g.meta["same_files"])
    r = subprocess.run([build.CLI, inp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"pairs in={g.n_in}" in r.stdout
    out = os.path.join(str(tmp_path), "out", "run_")
    for fname, ref in g.files.items():
        if fname.endswith(".info"):
            continue
        compare_files(open(out + fname).read(), ref, label=f"{name}:{fname}")
    # the run record: one entry per counted pair type
    rec = json.load(open(out + "run.json"))
    sd = [t for t in rec["terms"] if t["pair_type"] == "SD"]
    assert rec["engine"] == "fast" and len(sd) == 1
    assert sd[0]["n_binned"] == g.n_in and sd[0]["n_window"] == g.n_total
    assert sd[0]["kernel_ms"] > 0 and sd[0]["binned_pairs_per_s"] > 0


@pytest.mark.parametrize("name", ["sky_wgp_jk", "sky_wgg_distinct_wrap", "nbox_wgp_ls"])
def test_cli_sky_output_files_match_reference(name, tmp_path):
    """A sky cross run through the command line: reads the four catalogues and
    the distances file, counts SRd, RsRd, SD, DRs on the GPU, finalises with
    Landy-Szalay and writes the reference's files."""
    from helpers import SkyGolden
    g = SkyGolden(name)
    c = g.cats
    wl = synth.SkyWorkload(name, g.params, g.table, c["S"], c["D"], c["Rs"], c["Rd"])
    inp = synth.write_sky_run(str(tmp_path), wl, same_files=g.meta["same_files"])
    r = subprocess.run([build.CLI, inp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for t in g.terms:
        assert f"pairs in={g.term(t)[2]}" in r.stdout, t
    out = os.path.join(str(tmp_path), "out", "run_")
    rec = {t["pair_type"]: t for t in json.load(open(out + "run.json"))["terms"]}
    for t in g.terms:
        assert rec[t]["n_binned"] == g.term(t)[2], t
    for fname, ref in g.files.items():
        if fname.endswith(".info"):
            continue
        compare_files(open(out + fname).read(), ref, label=f"{name}:{fname}")


@pytest.mark.parametrize("name", ["auto_box_wgg", "auto_box_wpp_rebin", "auto_box_wgp_unsorted",
                                  "auto_sky_wgp", "auto_nbox_wgg", "auto_box_ed_rmu"])
def test_cli_auto_output_files_match_reference(name, tmp_path):
    """Auto-correlation runs (estimators 1 and 2) through the command line:
    corels1 on the GPU, final_calc_auto (re_bin for estimator 2), the
    reference's bins_auto_* files."""
    from helpers import AutoGolden
    g = AutoGolden(name)
    S = g.cats["S"]
    if g.table is None:
        inp = synth.write_box_run(str(tmp_path), synth.Workload(name, g.params, S, S),
                                  same_files=True)
    else:
        R = g.cats["Rs"]
        inp = synth.write_sky_run(str(tmp_path), synth.SkyWorkload(name, g.params, g.table, S, S,
                                                                   R, R))
    r = subprocess.run([build.CLI, inp], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for t in g.terms:
        assert f"pairs in={g.term(t)[2]}" in r.stdout, t
    out = os.path.join(str(tmp_path), "out", "run_")
    rec = {t["pair_type"]: t for t in json.load(open(out + "run.json"))["terms"]}
    for t in g.terms:
        assert rec[t]["n_binned"] == g.term(t)[2], t
    for fname, ref in g.files.items():
        if fname.endswith(".info"):
            continue
        compare_files(open(out + fname).read(), ref, label=f"{name}:{fname}")


def test_cli_batch_of_box_runs_matches_reference(tmp_path):
    """Three periodic-box runs (their own .inp, catalogues and output prefix)
    through one `--batch` call: their SD terms are counted in one launch and
    every run writes the reference's files."""
    names = ["box_wgg_uniform", "box_wgp_clustered", "box_wpp_weighted_distinct"]
    inps, outs, goldens = [], [], []
    for k, name in enumerate(names):
        g = Golden(name)
        d = tmp_path / f"run{k}"
        d.mkdir()
        wl = synth.Workload(name, g.params, g.S, g.D)
        inps.append(synth.write_box_run(str(d), wl, same_files=g.meta["same_files"]))
        outs.append(os.path.join(str(d), "out", "run_"))
        goldens.append(g)
    r = subprocess.run([build.CLI, "--batch", *inps], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for name, g, out in zip(names, goldens, outs):
        assert f"pairs in={g.n_in}" in r.stdout, name
        for fname, ref in g.files.items():
            if fname.endswith(".info"):
                continue
            compare_files(open(out + fname).read(), ref, label=f"batch {name}:{fname}")
        sd = [t for t in json.load(open(out + "run.json"))["terms"] if t["pair_type"] == "SD"]
        assert sd[0]["n_binned"] == g.n_in and sd[0]["n_window"] == g.n_total


def test_cli_batch_rejects_a_sky_run(tmp_path):
    from helpers import SkyGolden
    g = SkyGolden("sky_wgp_jk")
    c = g.cats
    wl = synth.SkyWorkload("sky_wgp_jk", g.params, g.table, c["S"], c["D"], c["Rs"], c["Rd"])
    inp = synth.write_sky_run(str(tmp_path), wl, same_files=g.meta["same_files"])
    r = subprocess.run([build.CLI, "--batch", inp], capture_output=True, text=True, timeout=600)
    assert r.returncode != 0 and "--batch takes periodic-box cross runs" in r.stdout
