"""Python host mirror of the reference's read path and pair-loop interface.

* ``prepare``  -- what ``read_data`` (read_dat.cpp:18-347) derives per galaxy
  before the pair loop: the jackknife draw ``jk_prob`` (glibc ``rand()`` after
  ``srand(124693517)``, one draw per galaxy in read order, read_dat.cpp:241-246),
  the orientation ``phi`` (elip_angle, read_dat.cpp:275-280) or -10, unit
  weights, the ``include_prob`` draw of random catalogues, and which samples
  read ellipticities, kappa or the ED orientation (read_dat.cpp:27-133).
* ``corels2``  -- the reference's ``long corels2(gal g1[], gal g2[], bin_jk&,
  data_info&)`` (corr.cpp:219-459) on the GPU: counts one pair type through the
  C ABI and returns the bin_jk contents after the delete-one conversion
  ``final_jk_bins`` (jk.cpp:74-81), plus ``n_in`` (its return value).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib

JK_SEED = 124693517  # jk.cpp:40-43
RAND_MAX = 2147483647


@dataclass
class Galaxies:
    """Flattened gal[] (data_def.h:23-44) as the pair loop reads it."""

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    w: np.ndarray
    e1: np.ndarray | None
    e2: np.ndarray | None
    phi: np.ndarray
    jk: np.ndarray | None
    jk_prob: np.ndarray
    include_prob: np.ndarray
    dc: np.ndarray | None = None  # sky: comoving distance (table row of z)
    da: np.ndarray | None = None  # sky: transverse distance (table row of z)
    e3: np.ndarray | None = None  # ED orientation e[2] (which_corr 5)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])


def e_columns(params, role: str):
    """What a sample's e file holds for the pair loop (read_dat.cpp:27-113):
    "e" (e1, e2; phi from elip_angle), "kappa" (one column stored as e[0]),
    "e3" (the 3-D ED orientation, normalised to unit length at read,
    read_dat.cpp:282-293) or None (nothing read).  which_corr 5 falls through
    into case 8 (read_dat.cpp:50-58), so its density sample reads nothing."""
    if role == "S":
        return {1: "e", 2: "e", 3: "kappa", 4: "e", 5: "e3"}.get(params.which_corr)
    if role == "D":
        return {2: "e", 4: "kappa"}.get(params.which_corr)
    return None


def reads_e(params, role: str) -> bool:
    """Whether a sample reads ellipticities e1, e2."""
    return e_columns(params, role) == "e"


def prepare(params, cats_in_read_order, table=None) -> dict:
    """cats_in_read_order: list of (role, catalogue with x,y,z[,w,e1,e2,jk]) in the
    order do_corr reads them (S, Rs, D, Rd; do_corr.cpp:40-96).  Sky runs pass
    the distance table: DC and DA are the table rows at floor(z/dz), without
    interpolation (read_dat.cpp:247-251)."""
    out = {}
    pos = 0
    for role, c in cats_in_read_order:
        n = int(np.asarray(c.x).shape[0])
        randoms = role in ("Rs", "Rd")
        draws = (1 if params.periodic_box else 0) + (1 if randoms else 0)
        r = _lib.rand_uniform(JK_SEED, pos, n * draws) if (draws and n) else np.zeros(0)
        if n:
            pos += n * draws
        jkp = np.ones(n)
        inc = np.zeros(n)
        if params.periodic_box and n:
            jkp = r[0::draws].copy()
            if randoms:
                inc = r[1::draws].copy()
        elif randoms and n:
            inc = r.copy()
        if params.do_jk == 0 or params.n_jk_regions == 0:
            jkp = np.zeros(n)
        mode = e_columns(params, role) if getattr(c, "e1", None) is not None else None
        e1 = e2 = e3 = None
        phi = np.full(n, -10.0)
        if mode == "e":
            e1 = np.ascontiguousarray(c.e1, dtype=np.float64)
            e2 = np.ascontiguousarray(c.e2, dtype=np.float64)
            phi = _lib.elip_angle(e1, e2)
        elif mode == "kappa":
            e1 = np.ascontiguousarray(c.e1, dtype=np.float64)
        elif mode == "e3":
            e1, e2, e3 = (np.array(v, dtype=np.float64) for v in (c.e1, c.e2, c.e3))
            norm = np.sqrt(e1 * e1 + e2 * e2 + e3 * e3)
            nz = norm > 0
            for v in (e1, e2, e3):
                v[nz] /= norm[nz]
        w = getattr(c, "w", None)
        w = np.ones(n) if w is None else np.ascontiguousarray(w, dtype=np.float64)
        jk = getattr(c, "jk", None) if params.do_jk else None
        dc = da = None
        if not params.periodic_box and table is not None:
            it = np.floor(np.asarray(c.z, dtype=np.float64) / params.dz).astype(np.int64)
            dc = np.ascontiguousarray(table.DC[it])
            da = np.ascontiguousarray((table.transverse if params.use_comoving else table.DA)[it])
        out[role] = Galaxies(np.ascontiguousarray(c.x, dtype=np.float64),
                             np.ascontiguousarray(c.y, dtype=np.float64),
                             np.ascontiguousarray(c.z, dtype=np.float64), w, e1, e2, phi,
                             None if jk is None else np.ascontiguousarray(jk, dtype=np.int32),
                             jkp, inc, dc, da, e3)
    return out


def delete_one(num: np.ndarray, sums: np.ndarray):
    """final_jk_bins (jk.cpp:74-81): jk[r] := full - region[r] for every field."""
    n2 = num.copy()
    s2 = sums.copy()
    n2[1:] = num[0][None] - num[1:]
    s2[1:] = sums[0][None] - sums[1:]
    return n2, s2


def corels2(ctx: "_lib.Context", kind: str, slot_g1: int, slot_g2: int, *,
            engine: str = "fast") -> dict:
    """GPU corels2 for one pair type.  Returns the p_bin arrays after the
    delete-one conversion (h = 0 full sample, h = 1 + r jackknife sample r),
    the 1-D r_p counts, and n_in (the reference's return value)."""
    r = ctx.count(kind, slot_g1, slot_g2, engine=engine)
    num, sums = r["num"], r["sums"]
    if ctx.params.do_jk:
        num, sums = delete_one(num, sums)
    return {"p_num": num, "p_sums": sums, "b_num": num.sum(axis=2), "n_in": r["n_binned"],
            "n_total": r["n_window"], "kernel_ms": r["kernel_ms"],
            "n_rechecked": r["n_rechecked"]}
