"""Test helpers: golden fixtures and tolerance checks."""
from __future__ import annotations

import glob
import json
import os

import numpy as np

from corr_pc_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_names():
    """Periodic-box fixtures (one SD term each)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "box_*.npz")))


def sky_golden_names():
    """Cross runs with randoms and a distances table (four terms each: SRd, RsRd,
    SD, DRs): the sky fixtures and the box without periodic images."""
    return sorted(os.path.basename(p)[:-4] for pat in ("sky_*.npz", "nbox_*.npz")
                  for p in glob.glob(os.path.join(GOLDEN, pat)))


def auto_golden_names():
    """Auto-correlation fixtures (estimator 1/2: SS by corels1; the sky also SRs
    by corels2 and RsRs by corels1)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "auto_*.npz")))


class AutoGolden:
    """An auto-correlation run as the reference computed it."""

    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
        self.meta = json.loads(str(z["meta"]))
        self.arr = {k: z[k] for k in z.files if k != "meta"}
        p = synth.InpParams()
        for k, v in self.meta["params"].items():
            setattr(p, k, v)
        self.params = p
        a = self.arr
        self.table = None
        if "table_H" in a:
            self.table = synth.DistanceTable(p.dz * np.arange(a["table_H"].shape[0]),
                                             a["table_H"], a["table_DA"], a["table_DC"])
        self.cats = {}
        for r in ("S", "Rs"):
            if f"{r}_x" in a:
                g = lambda q: a.get(f"{r}_{q}")
                self.cats[r] = synth.Catalog(g("x"), g("y"), g("z"), g("w"), g("e1"), g("e2"),
                                             g("jk"), g("e3"))
        self.terms = self.meta["terms"]
        self.files = self.meta["files"]

    def read_order(self):
        return [(r, self.cats[r]) for r in ("S", "Rs") if r in self.cats]

    def term(self, t):
        a = self.arr
        return (a[f"{t}_raw_num"], a[f"{t}_raw_sums"], int(a[f"{t}_n_in"]),
                int(a[f"{t}_n_total"]))


class SkyGolden:
    """A cross run with randoms (sky, or a box without periodic images) as the
    reference computed it: four catalogues, the distances table and, per term,
    the raw histograms and pair counters.  The
    reference's DRs term was run as a density-density count (its wg+ DRs term
    crashes), so only its counts and weights are compared."""

    KIND = {"SRd": ("SRd", "Rd", "S"), "RsRd": ("RsRd", "Rd", "Rs"), "SD": ("SD", "D", "S"),
            "DRs": ("DRs", "Rs", "D")}

    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
        self.meta = json.loads(str(z["meta"]))
        self.arr = {k: z[k] for k in z.files if k != "meta"}
        p = synth.InpParams()
        for k, v in self.meta["params"].items():
            setattr(p, k, v)
        self.params = p
        a = self.arr
        self.table = synth.DistanceTable(p.dz * np.arange(a["table_H"].shape[0]), a["table_H"],
                                         a["table_DA"], a["table_DC"])
        self.cats = {r: self._cat(r) for r in ("S", "D", "Rs", "Rd")}
        self.terms = self.meta["terms"]
        self.files = self.meta["files"]

    def _cat(self, role):
        g = lambda a: self.arr.get(f"{role}_{a}")
        return synth.Catalog(g("x"), g("y"), g("z"), g("w"), g("e1"), g("e2"), g("jk"), g("e3"))

    def read_order(self):
        return [(r, self.cats[r]) for r in ("S", "Rs", "D", "Rd")]

    def term(self, t):
        a = self.arr
        return (a[f"{t}_raw_num"], a[f"{t}_raw_sums"], int(a[f"{t}_n_in"]),
                int(a[f"{t}_n_total"]))


class Golden:
    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
        self.meta = json.loads(str(z["meta"]))
        self.arr = {k: z[k] for k in z.files if k != "meta"}
        p = synth.InpParams()
        for k, v in self.meta["params"].items():
            setattr(p, k, v)
        self.params = p
        self.S = self._cat("S")
        self.D = self._cat("D")
        self.raw_num = self.arr["raw_num"]
        self.raw_sums = self.arr["raw_sums"]
        self.n_in = int(self.arr["n_in"])
        self.n_total = int(self.arr["n_total"])
        self.files = self.meta["files"]

    def _cat(self, role):
        g = lambda a: self.arr.get(f"{role}_{a}")
        return synth.Catalog(g("x"), g("y"), g("z"), g("w"), g("e1"), g("e2"), g("jk"), g("e3"))

    def weights(self):
        w = []
        for c in (self.S, self.D):
            ww = np.ones(c.n) if c.w is None else c.w
            w += [float(ww.sum()), float((ww * ww).sum())]
        return w + [0.0, 0.0, 0.0, 0.0]


def check_sums(got, ref, rtol=1e-6, label="", big_frac=1e-2):
    """Accuracy bar, for every field (the cancelling e+/ex and product sums
    included): bins holding at least big_frac of the field's largest |value|
    within rtol relative; the other bins, whose true value is near zero, within
    rtol x that largest value; and the Pi-integrated r_p profile of the full
    sample (the w(r_p) numerator) within rtol relative wherever it holds at
    least big_frac of its largest value."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    for f in range(ref.shape[-1]):
        r = ref[..., f]
        g = got[..., f]
        fmax = np.abs(r).max()
        if fmax == 0:
            assert np.abs(g).max() == 0, f"{label} field {f}: expected zeros"
            continue
        err = np.abs(g - r)
        assert err.max() <= rtol * fmax, f"{label} field {f}: max err {err.max()} vs floor {rtol * fmax}"
        big = np.abs(r) >= big_frac * fmax
        rel = err[big] / np.abs(r[big])
        assert rel.max() <= rtol, f"{label} field {f}: per-bin rel err {rel.max()}"
        if r.ndim == 3:  # [histogram, r_p, Pi]: the full sample's r_p profile
            pr, pg = r[0].sum(axis=-1), g[0].sum(axis=-1)
            pmax = np.abs(pr).max()
            if pmax > 0:
                pb = np.abs(pr) >= big_frac * pmax
                prel = np.abs(pg - pr)[pb] / np.abs(pr[pb])
                assert prel.max() <= rtol, f"{label} field {f}: r_p profile rel err {prel.max()}"


def parse_table(text):
    """Numeric tokens of an output file (header skipped); nan/-nan -> nan."""
    rows = []
    for line in text.splitlines():
        if not line.strip() or line.startswith("#"):
            continue
        rows.append([float(t.replace("-nan", "nan")) for t in line.split()])
    return rows


def compare_files(got_text, ref_text, rtol=2e-5, label=""):
    """Numbers are printed with 6 significant digits: allow last-digit rounding
    (rtol) per value, and 1e-6 of the column's largest value for entries that
    are themselves tiny results of cancellation."""
    a, b = parse_table(got_text), parse_table(ref_text)
    assert len(a) == len(b), f"{label}: {len(a)} rows vs {len(b)}"
    a = np.array(a, dtype=np.float64)
    b = np.array(b, dtype=np.float64)
    assert a.shape == b.shape, f"{label}: shape {a.shape} vs {b.shape}"
    nan_b = np.isnan(b)
    assert np.array_equal(np.isnan(a), nan_b), f"{label}: nan pattern differs"
    colmax = np.nanmax(np.where(nan_b, 0, np.abs(b)), axis=0)
    d = np.abs(np.where(nan_b, 0, a - b))
    ok = (d <= rtol * np.abs(np.where(nan_b, 0, b))) | (d <= 1e-6 * colmax[None, :])
    bad = np.argwhere(~ok)
    assert bad.size == 0, f"{label}: {len(bad)} values differ, first at {bad[0]}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}"
