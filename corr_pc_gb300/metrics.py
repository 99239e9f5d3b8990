"""Algorithmic work per binned pair -- the constants the benchmark's roofline
fractions use (one place, shared by bench.py and the docs).

FP32 flops per binned pair (separation and r_p^2: 3 sub + 2 mul + 1 add = 6;
weight product 1):
  wgg  F = 7
  wg+  F = 33  (+ raw dx', dy' 2; cos 2theta / sin 2theta from (dx'^2 - dy'^2)/q,
                2dx'dy'/q 8; two-component rotation 6; w e, (w e)^2 for e+ and
                ex 4; theta term ~4; tally 2)
  w++  F = 55  (+ second rotation 6, three products and their squares 12, less reuse)
  kappa-density (which_corr 3)  F = 8   (wgg + w kappa)
  shape-kappa   (which_corr 4)  F = 26  (wgg + angle 10, rotation 6, w kappa and
                                         its two products 3)
  ED            (which_corr 5)  F = 17  (wgg + dz^2 2, orientation dot product 5,
                                         its square over r^2 2, the square 1)
  r-mu binning (coordinates 7) adds 4: dz^2 into r^2, sqrt, mu = dz / r.
Shared-memory atomic updates per binned pair (main fields M + jackknife fields
J per attribution; one attribution per pair on average in a periodic box):
  wgg  M = 3,  J = 3
  wg+  M = 9,  J = 6
  w++  M = 15, J = 9
  kappa M = 4, J = 4;  shape-kappa M = 6, J = 6;  ED M = 5, J = 4
"""

FLOPS_PER_PAIR = {0: 7, 1: 33, 2: 55, 3: 8, 4: 26, 5: 17}
RMU_EXTRA_FLOPS = 4
SMEM_MAIN = {0: 3, 1: 9, 2: 15, 3: 4, 4: 6, 5: 5}
SMEM_JK = {0: 3, 1: 6, 2: 9, 3: 4, 4: 6, 5: 4}


def flops_per_pair(which_corr: int, coordinates: int = 6) -> int:
    return FLOPS_PER_PAIR[which_corr] + (RMU_EXTRA_FLOPS if coordinates == 7 else 0)


def smem_updates_per_pair(which_corr: int, do_jk: bool, attributions: float = 1.0) -> float:
    return SMEM_MAIN[which_corr] + (attributions * SMEM_JK[which_corr] if do_jk else 0.0)


# histogram fields (cpc_accum layout): p_bin.wt_num, then data[1..6].val/.err
FIELD_NAMES = ["wt_num"] + [f"data{j}.{v}" for j in range(1, 7) for v in ("val", "err")]
# fields whose per-pair terms cannot cancel (weights, squares, the theta term)
NONCANCEL = (0, 2, 4, 6, 8, 10, 11, 12)


def accuracy_report(num, sums, ref_num, ref_sums, rtol: float = 1e-6, big_frac: float = 1e-2):
    """Per-bin error of a histogram block against a double-precision one of the
    same rows: whether every integer count (full sample and every jackknife
    region) is identical, and per field the largest |error| over all bins as a
    fraction of the field's largest |value|, the largest relative error over the
    bins holding at least `big_frac` of that value, and the largest relative
    error of the Pi-integrated r_p profile (sum over Pi bins, full sample: the
    numerator of w(r_p)) over the profile entries holding at least `big_frac`
    of the profile's largest value.  `ok` applies the bar to every field,
    cancelling sums included: counts identical; bins and profile entries holding
    >= big_frac of the field's largest value within rtol relative; the other
    bins (whose true value is near zero) within rtol x the field's largest
    value."""
    import numpy as np
    num, ref_num = np.asarray(num), np.asarray(ref_num)
    sums, ref_sums = np.asarray(sums, dtype=np.float64), np.asarray(ref_sums, dtype=np.float64)
    out = {"counts_bit_exact": bool(np.array_equal(num, ref_num)),
           "n_bins_compared": int(ref_num.size), "fields": {}}
    ok = out["counts_bit_exact"]
    for f in range(ref_sums.shape[-1]):
        r, g = ref_sums[..., f], sums[..., f]
        fmax = float(np.abs(r).max()) if r.size else 0.0
        if fmax == 0.0:
            if r.size and float(np.abs(g).max()) != 0.0:
                ok = False
            continue
        err = np.abs(g - r)
        big = np.abs(r) >= big_frac * fmax
        rel_big = float((err[big] / np.abs(r[big])).max())
        pr, pg = r[0].sum(axis=-1), g[0].sum(axis=-1)  # full sample, summed over Pi
        pmax = float(np.abs(pr).max())
        pbig = np.abs(pr) >= big_frac * pmax
        prof = float((np.abs(pg - pr)[pbig] / np.abs(pr[pbig])).max()) if pmax > 0 else 0.0
        e_floor = float(err.max()) / fmax
        out["fields"][FIELD_NAMES[f]] = {"max_err_over_field_max": e_floor,
                                         "max_rel_err_bins_ge_1pct": rel_big,
                                         "max_rel_err_rp_profile": prof,
                                         "cancelling": f not in NONCANCEL}
        ok = ok and e_floor <= rtol and rel_big <= rtol and prof <= rtol
    out["ok"] = bool(ok)
    out["bar"] = (f"counts identical; every field (cancelling sums included) <= {rtol:g} "
                  f"relative in bins and r_p profile entries holding >= {big_frac:g} of its "
                  f"largest value, <= {rtol:g} x that value elsewhere")
    return out
