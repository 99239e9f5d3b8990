"""Python access to the oracle.  TEST INFRASTRUCTURE ONLY.

Imported only by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline arm, and only as the checker / the timed CPU baseline -- never by the
product path.

* ``port_corels2``   -- the plain-C restatement of ``corels2`` (cpc_oracle.c).
* ``read_like_reference`` -- per-galaxy attributes the reference derives at read
  time (read_dat.cpp:216-325): jackknife draws ``jk_prob`` from glibc
  ``rand()`` after ``srand(124693517)`` in read order, ``phi`` from
  ``elip_angle`` (calcs.cpp:73-83), weights and labels.
* ``run_reference`` / ``parse_dump`` -- the reference itself, built from its
  own sources by oracle/Makefile into oracle/_ref (only where the reference
  tree exists).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# CPC_ORACLE_SO: another build of the restatement (the sanitizer test's)
PORT_SO = os.environ.get("CPC_ORACLE_SO") or os.path.join(HERE, "_build", "libcpc_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_harness")
NF = 13  # wt, d1v, d1e, ..., d6v, d6e
KIND = {"SD": 0, "SRd": 1, "DRs": 2, "RsRd": 3, "RsRs": 4, "SRs": 5, "SS": 6}
JK_SEED = 124693517  # jk.cpp:40-43
RAND_MAX = 2147483647


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_SO


# the reference tree (read-only): CPC_REFERENCE_DIR, else its usual place here
REF_DIR = os.environ.get("CPC_REFERENCE_DIR", "/root/reference")


def build_reference() -> str | None:
    """Build the reference harness from the reference sources (no-op where the
    reference tree is absent)."""
    if not os.path.isdir(REF_DIR):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_DIR}"], check=True)
    return REF_BIN


class _Cat(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [
        (nm, ctypes.c_void_p) for nm in
        ("x", "y", "z", "w", "e1", "e2", "phi", "jk", "jk_prob", "include_prob", "dc", "da",
         "e3")]


class _Params(ctypes.Structure):
    _fields_ = [(nm, ctypes.c_int) for nm in
                ("which_corr", "coordinates", "estimator", "periodic_box", "data_sorted",
                 "do_jk", "n_jk", "lin_bin", "n_bins", "n_p_bin", "sig_crit")] + [
        (nm, ctypes.c_double) for nm in
        ("bin_r_min", "bin_r_max", "p_min", "p_max", "box", "include_prob_rr",
         "z_max_data", "dz", "z_sep_max")] + [
        ("H_z", ctypes.c_void_p), ("dA_z", ctypes.c_void_p), ("n_table", ctypes.c_int64),
        ("n_threads", ctypes.c_int), ("row_stride", ctypes.c_int64),
        ("row_offset", ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(PORT_SO):
            build_port()
        _lib = ctypes.CDLL(PORT_SO)
        _lib.orc_corels2.restype = ctypes.c_int
        _lib.orc_corels2.argtypes = [ctypes.POINTER(_Params), ctypes.c_int,
                                     ctypes.POINTER(_Cat), ctypes.POINTER(_Cat),
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib.orc_corels1.restype = ctypes.c_int
        _lib.orc_corels1.argtypes = [ctypes.POINTER(_Params), ctypes.c_int,
                                     ctypes.POINTER(_Cat), ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p]
        _lib.orc_elip_angle.restype = None
        _lib.orc_elip_angle.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]
        _lib.orc_glibc_rand.restype = None
        _lib.orc_glibc_rand.argtypes = [ctypes.c_uint32, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_void_p]
    return _lib


def glibc_rand(seed: int, skip: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.int32)
    lib().orc_glibc_rand(seed, skip, n, out.ctypes.data)
    return out


def _ptr(a):
    return None if a is None else a.ctypes.data


class OracleCatalog:
    """A catalogue with the per-galaxy attributes the pair loop reads."""

    def __init__(self, x, y, z, *, w=None, e1=None, e2=None, phi=None, jk=None,
                 jk_prob=None, include_prob=None, dc=None, da=None, e3=None):
        f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        self.x, self.y, self.z = f(x), f(y), f(z)
        self.w, self.e1, self.e2, self.phi = f(w), f(e1), f(e2), f(phi)
        self.e3 = f(e3)
        self.jk = None if jk is None else np.ascontiguousarray(jk, dtype=np.int32)
        self.jk_prob, self.include_prob = f(jk_prob), f(include_prob)
        self.dc, self.da = f(dc), f(da)
        self.n = int(self.x.shape[0])

    def cstruct(self) -> _Cat:
        c = _Cat()
        c.n = self.n
        for nm in ("x", "y", "z", "w", "e1", "e2", "phi", "jk", "jk_prob",
                   "include_prob", "dc", "da", "e3"):
            setattr(c, nm, _ptr(getattr(self, nm)))
        return c


def elip_angle(e1, e2):
    """phi = 0.5*arctan(e1, -e2) with the reference's quadrant rule
    (calcs.cpp:35-46, 73-83); NaN -> 0.  Evaluated in C with the C library's
    atan, as the reference does."""
    e1 = np.ascontiguousarray(e1, dtype=np.float64)
    e2 = np.ascontiguousarray(e2, dtype=np.float64)
    out = np.empty_like(e1)
    lib().orc_elip_angle(e1.shape[0], e1.ctypes.data, e2.ctypes.data, out.ctypes.data)
    return out


def e_columns(which_corr, role):
    """What read_data reads from a sample's e file (read_dat.cpp:27-113):
    "e" (e1 e2, then elip_angle), "kappa" (one column into e[0]), "e3" (three
    columns, normalised to unit length, read_dat.cpp:282-293) or None.  Note the
    fall-through of which_corr 5 into case 8 (read_dat.cpp:50-58): the density
    sample reads nothing there."""
    if role == "S":
        return {1: "e", 2: "e", 3: "kappa", 4: "e", 5: "e3"}.get(which_corr)
    if role == "D":
        return {2: "e", 4: "kappa"}.get(which_corr)
    return None


def read_like_reference(params, cats_in_read_order, table=None):
    """Attach jk_prob / phi / include_prob as read_data does, consuming one glibc
    rand() stream across the catalogues in the reference's read order.

    ``cats_in_read_order``: list of (role, Catalog-like with x,y,z,w,e1,e2,jk)
    with role in {"S", "Rs", "D", "Rd"}.  Returns dict role -> OracleCatalog.
    ``table`` (sky runs): the distances table (z, H, DA, DC rows); each galaxy
    gets DC = D_C[floor(z/dz)] and DA = the transverse column at the same row,
    without interpolation (read_dat.cpp:247-251; use_comoving 1 stores the
    table's fifth column as D_A, initialization.cpp:40-44).
    """
    p = params
    pos = 0
    out = {}
    for role, c in cats_in_read_order:
        n = c.x.shape[0]
        if n == 0:
            out[role] = OracleCatalog(c.x, c.y, c.z)
            continue
        randoms = role in ("Rs", "Rd")
        draws_per = (1 if p.periodic_box else 0) + (1 if randoms else 0)
        r = glibc_rand(JK_SEED, pos, n * draws_per).astype(np.float64) if draws_per else None
        pos += n * draws_per
        jkp = np.ones(n)
        inc = np.zeros(n)
        if p.periodic_box:
            jkp = r[0::draws_per] / (RAND_MAX + 1.0)
            if randoms:
                inc = r[1::draws_per] / (RAND_MAX + 1.0)
        elif randoms:
            inc = r / (RAND_MAX + 1.0)
        if p.do_jk == 0 or p.n_jk_regions == 0:
            jkp = np.zeros(n)
        mode = e_columns(p.which_corr, role) if getattr(c, "e1", None) is not None else None
        e1 = e2 = e3 = None
        phi = np.full(n, -10.0)
        if mode == "e":
            e1, e2 = c.e1, c.e2
            phi = elip_angle(e1, e2)
        elif mode == "kappa":
            e1 = c.e1
        elif mode == "e3":
            a, b, d = (np.asarray(v, dtype=np.float64) for v in (c.e1, c.e2, c.e3))
            nrm = np.sqrt(a * a + b * b + d * d)
            nz = nrm > 0
            e1, e2, e3 = a.copy(), b.copy(), d.copy()
            e1[nz] /= nrm[nz]
            e2[nz] /= nrm[nz]
            e3[nz] /= nrm[nz]
        w = c.w if c.w is not None else np.ones(n)
        jk = c.jk if (p.do_jk and c.jk is not None) else None
        dc = da = None
        if not p.periodic_box:
            it = np.floor(np.asarray(c.z) / p.dz).astype(np.int64)
            dc = table.DC[it]
            da = (table.transverse if p.use_comoving else table.DA)[it]
        out[role] = OracleCatalog(c.x, c.y, c.z, w=w, e1=e1, e2=e2, phi=phi, jk=jk,
                                  jk_prob=jkp, include_prob=inc, dc=dc, da=da, e3=e3)
    return out


def _params_struct(p, n_threads, row_stride, row_offset, H_z, dA_z, z_sep_max):
    P = _Params()
    P.which_corr, P.coordinates, P.estimator = p.which_corr, p.coordinates, p.estimator
    P.periodic_box, P.data_sorted, P.do_jk = int(p.periodic_box), p.data_sorted, p.do_jk
    P.n_jk, P.lin_bin, P.n_bins, P.n_p_bin = p.n_jk_regions, int(p.lin_bin), p.n_bins, p.n_p_bin
    P.sig_crit = p.sig_crit
    P.bin_r_min, P.bin_r_max, P.p_min, P.p_max = p.bin_r_min, p.bin_r_max, p.p_min, p.p_max
    P.box = p.periodic_box_size
    P.include_prob_rr = 1.0
    P.z_max_data, P.dz = p.z_max, p.dz
    P.z_sep_max = p.z_sep_max if z_sep_max is None else z_sep_max
    keep = []
    if H_z is not None:
        H_z = np.ascontiguousarray(H_z, dtype=np.float64)
        dA_z = np.ascontiguousarray(dA_z, dtype=np.float64)
        keep += [H_z, dA_z]
        P.H_z, P.dA_z, P.n_table = H_z.ctypes.data, dA_z.ctypes.data, H_z.shape[0]
    P.n_threads, P.row_stride, P.row_offset = n_threads, row_stride, row_offset
    return P, keep


def port_corels1(params, kind: str, g: OracleCatalog, *, n_threads: int = 0,
                 row_stride: int = 1, row_offset: int = 0, H_z=None, dA_z=None,
                 z_sep_max: float | None = None):
    """The C restatement of corels1 (auto pairs of one catalogue); kind "SS"
    (do_SS) or "RsRs" (do_RsRs).  Same return values as port_corels2."""
    p = params
    P, keep = _params_struct(p, n_threads, row_stride, row_offset, H_z, dA_z, z_sep_max)
    n_hist = 1 + (p.n_jk_regions if p.do_jk else 0)
    num = np.zeros((n_hist, p.n_bins, p.n_p_bin), dtype=np.int64)
    sums = np.zeros((n_hist, p.n_bins, p.n_p_bin, NF), dtype=np.float64)
    cnt = np.zeros(2, dtype=np.int64)
    cg = g.cstruct()
    rc = lib().orc_corels1(ctypes.byref(P), KIND[kind], ctypes.byref(cg), num.ctypes.data,
                           sums.ctypes.data, cnt.ctypes.data)
    if rc != 0:
        raise ValueError(f"orc_corels1 failed with code {rc}")
    return num, sums, int(cnt[0]), int(cnt[1])


def port_corels2(params, kind: str, ga: OracleCatalog, gb: OracleCatalog, *,
                 n_threads: int = 0, row_stride: int = 1, row_offset: int = 0,
                 H_z=None, dA_z=None, z_sep_max: float | None = None):
    """Run the C restatement of corels2 for one pair type.  Returns
    (num[h,i,k] int64, sums[h,i,k,NF] float64, n_total, n_in) with RAW region
    sums (h = 0 full, 1 + r region r)."""
    p = params
    P = _Params()
    P.which_corr, P.coordinates, P.estimator = p.which_corr, p.coordinates, p.estimator
    P.periodic_box, P.data_sorted, P.do_jk = int(p.periodic_box), p.data_sorted, p.do_jk
    P.n_jk, P.lin_bin, P.n_bins, P.n_p_bin = p.n_jk_regions, int(p.lin_bin), p.n_bins, p.n_p_bin
    P.sig_crit = p.sig_crit
    P.bin_r_min, P.bin_r_max, P.p_min, P.p_max = p.bin_r_min, p.bin_r_max, p.p_min, p.p_max
    P.box = p.periodic_box_size
    P.include_prob_rr = 1.0
    P.z_max_data, P.dz = p.z_max, p.dz
    P.z_sep_max = p.z_sep_max if z_sep_max is None else z_sep_max
    keep = []
    if H_z is not None:
        H_z = np.ascontiguousarray(H_z, dtype=np.float64)
        dA_z = np.ascontiguousarray(dA_z, dtype=np.float64)
        keep += [H_z, dA_z]
        P.H_z, P.dA_z, P.n_table = H_z.ctypes.data, dA_z.ctypes.data, H_z.shape[0]
    P.n_threads, P.row_stride, P.row_offset = n_threads, row_stride, row_offset
    n_hist = 1 + (p.n_jk_regions if p.do_jk else 0)
    num = np.zeros((n_hist, p.n_bins, p.n_p_bin), dtype=np.int64)
    sums = np.zeros((n_hist, p.n_bins, p.n_p_bin, NF), dtype=np.float64)
    cnt = np.zeros(2, dtype=np.int64)
    ca, cb = ga.cstruct(), gb.cstruct()
    rc = lib().orc_corels2(ctypes.byref(P), KIND[kind], ctypes.byref(ca), ctypes.byref(cb),
                           num.ctypes.data, sums.ctypes.data, cnt.ctypes.data)
    if rc != 0:
        raise ValueError(f"orc_corels2 failed with code {rc}")
    return num, sums, int(cnt[0]), int(cnt[1])


# ---------------------------------------------------------------------------
# the reference itself (where built)
# ---------------------------------------------------------------------------


def reference_available() -> bool:
    return os.path.exists(REF_BIN)


def run_reference(inp: str, dump: str, *, bining: bool = True, timeout: float = 3600,
                  drs_wgg: bool = False):
    args = [REF_BIN, inp, dump] + ([] if bining else ["--no-bining"]) + \
        (["--drs-wgg"] if drs_wgg else [])
    r = subprocess.run(args, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference harness failed: {r.stdout[-2000:]} {r.stderr[-2000:]}")
    totals = []
    for line in r.stdout.splitlines():
        if "total pair=" in line:
            t = float(line.split("time:")[1].split()[0]) if "time:" in line else float("nan")
            n_tot = int(line.split("total pair=")[1].split()[0])
            totals.append((n_tot, t))
    return totals, r.stdout


def parse_dump(path: str) -> dict:
    """Parse the harness dump into per-term arrays.  The jackknife histograms in
    the dump are delete-one samples (full - region); ``raw`` recovers the
    region sums."""
    terms = {}
    cur = None
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "T":
                name, n_in, nb, npb, njk = t[1], int(t[2]), int(t[3]), int(t[4]), int(t[5])
                cur = {"n_in": n_in, "num": np.zeros((njk + 1, nb, npb), np.int64),
                       "sums": np.zeros((njk + 1, nb, npb, NF)),
                       "bnum": np.zeros((njk + 1, nb), np.int64),
                       "bsums": np.zeros((njk + 1, nb, 15))}
                terms[name] = cur
            elif t[0] == "B":
                h, i = int(t[1]), int(t[2])
                cur["bnum"][h, i] = int(t[3])
                cur["bsums"][h, i] = [float(v) for v in t[4:19]]
            elif t[0] == "P":
                h, i, k = int(t[1]), int(t[2]), int(t[3])
                cur["num"][h, i, k] = int(t[4])
                vals = [float(v) for v in t[5:20]]  # wt, d0v, d0e, d1v, ... d6e
                cur["sums"][h, i, k, 0] = vals[0]
                cur["sums"][h, i, k, 1:] = vals[3:]
            elif t[0] == "W":
                pass
    for term in terms.values():
        full_n, full_s = term["num"][0], term["sums"][0]
        term["raw_num"] = term["num"].copy()
        term["raw_sums"] = term["sums"].copy()
        term["raw_num"][1:] = full_n[None] - term["num"][1:]
        term["raw_sums"][1:] = full_s[None] - term["sums"][1:]
    return terms
