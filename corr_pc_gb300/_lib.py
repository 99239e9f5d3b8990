"""ctypes binding of the C ABI in include/corrpc.h (libcorrpc_gb300.so).

The library is built in-tree by ``corr_pc_gb300.build``.  Loading fails loudly
when it is missing: there is no CPU fallback for the pair loop.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libcorrpc_gb300.so")

# cpc_status
CPC_OK = 0
STATUS_NAMES = {0: "CPC_OK", 1: "CPC_ERR_INVALID", 2: "CPC_ERR_CUDA", 3: "CPC_ERR_NOMEM",
                4: "CPC_ERR_TIMEOUT", 5: "CPC_ERR_STATE", 6: "CPC_ERR_RANGE",
                7: "CPC_ERR_NODEVICE", 8: "CPC_ERR_HOST"}
# cpc_pair_kind (the data_info.do_* flag of each corels2 call)
PAIR = {"SD": 0, "SRd": 1, "DRs": 2, "RsRd": 3, "RsRs": 4, "SRs": 5, "SS": 6}
ENGINE = {"fast": 0, "fp64": 1, "cell_fp64": 2}
NF = 13

EXPORTED = ["cpc_version", "cpc_create", "cpc_destroy", "cpc_last_error", "cpc_upload",
            "cpc_count", "cpc_accum_shape", "cpc_count_batch", "cpc_set_tuning",
            "cpc_host_rand_uniform", "cpc_host_elip_angle", "cpc_host_rp_thresholds",
            "cpc_host_pi_thresholds", "cpc_launch_count", "cpc_host_finalize_cross",
            "cpc_count_fp64_noalloc"]


class CpcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class cpc_params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "which_corr", "coordinates", "estimator", "periodic_box", "data_sorted", "do_jk",
        "n_jk", "sig_crit", "rand_subsample", "n_bins", "lin_bin", "n_p_bin")] + [
        (n, ctypes.c_double) for n in (
            "bin_r_min", "bin_r_max", "p_min", "p_max", "periodic_box_size", "z_max", "dz",
            "z_sep_max")] + [
        ("H_z", ctypes.c_void_p), ("dA_z", ctypes.c_void_p), ("n_table", ctypes.c_int64)]


class cpc_catalog(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [(n, ctypes.c_void_p) for n in (
        "x", "y", "z", "w", "e1", "e2", "phi", "jk", "jk_prob", "dc", "da", "e3")]


class cpc_device_catalog(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [(n, ctypes.c_void_p) for n in (
        "x", "y", "z", "w", "e1", "e2", "phi", "jk", "jk_prob")]


class cpc_accum(ctypes.Structure):
    _fields_ = [("num", ctypes.c_void_p), ("sums", ctypes.c_void_p),
                ("n_window", ctypes.c_int64), ("n_binned", ctypes.c_int64),
                ("n_rechecked", ctypes.c_int64), ("kernel_ms", ctypes.c_double),
                ("pair_kernel_ms", ctypes.c_double)]


_lib = None


def load() -> ctypes.CDLL:
    """Load libcorrpc_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -m corr_pc_gb300.build` "
                          "(the GPU pair loop has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    P, V, I64, I = ctypes.POINTER, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    lib.cpc_version.restype = ctypes.c_char_p
    lib.cpc_last_error.restype = ctypes.c_char_p
    lib.cpc_last_error.argtypes = [V]
    lib.cpc_create.argtypes = [P(V), P(cpc_params)]
    lib.cpc_destroy.argtypes = [V]
    lib.cpc_upload.argtypes = [V, I, P(cpc_catalog)]
    lib.cpc_count.argtypes = [V, I, I, I, I, I64, I64, P(cpc_accum)]
    lib.cpc_count_auto.argtypes = [V, I, I, I, I64, I64, P(cpc_accum)]
    lib.cpc_count_async.argtypes = [V, I, I, I, I, I64, I64, V]
    lib.cpc_count_finish.argtypes = [V, P(cpc_accum)]
    lib.cpc_accum_shape.argtypes = [V, P(I), P(I), P(I)]
    lib.cpc_count_batch.argtypes = [I, P(V), P(I), P(I), P(I), P(cpc_accum)]
    lib.cpc_set_tuning.argtypes = [V, I, I, I]
    lib.cpc_autotune.argtypes = [V, I, I, I, I64, P(I), P(I)]
    lib.cpc_autotune_batch.argtypes = [I, P(V), P(I), P(I), P(I), I64, P(I), P(I)]
    lib.cpc_autotune.restype = I
    lib.cpc_host_rand_uniform.argtypes = [ctypes.c_uint32, I64, I64, V]
    lib.cpc_host_elip_angle.argtypes = [I64, V, V, V]
    lib.cpc_host_rp_thresholds.argtypes = [P(cpc_params), V]
    lib.cpc_host_pi_thresholds.argtypes = [P(cpc_params), V]
    lib.cpc_launch_count.argtypes = [V, P(I64)]
    lib.cpc_set_graph_replay.argtypes = [V, I]
    lib.cpc_set_shard.argtypes = [V, I, I]
    lib.cpc_graph_stats.argtypes = [V, P(I64), P(I64)]
    lib.cpc_set_twin.argtypes = [V, I]
    lib.cpc_last_twin.argtypes = [V, P(I)]
    lib.cpc_host_finalize_cross.argtypes = [ctypes.c_char_p] + [V] * 9
    lib.cpc_host_finalize_auto.argtypes = [ctypes.c_char_p] + [V] * 7
    lib.cpc_host_finalize_auto.restype = I
    lib.cpc_count_fp64_noalloc.argtypes = [P(cpc_params), I, P(cpc_device_catalog),
                                           P(cpc_device_catalog), V, V, P(I64), P(I64), V,
                                           ctypes.c_char_p, ctypes.c_size_t]
    lib.cpc_count_fp64_noalloc.restype = I
    for fn in ("cpc_create", "cpc_destroy", "cpc_upload", "cpc_count", "cpc_count_auto",
               "cpc_accum_shape",
               "cpc_count_batch", "cpc_set_tuning", "cpc_host_rand_uniform",
               "cpc_host_elip_angle", "cpc_host_rp_thresholds", "cpc_host_pi_thresholds",
               "cpc_launch_count", "cpc_host_finalize_cross", "cpc_set_graph_replay",
               "cpc_graph_stats", "cpc_set_shard", "cpc_set_twin", "cpc_last_twin"):
        getattr(lib, fn).restype = I
    _lib = lib
    return lib


def check(status: int, ctx=None) -> None:
    if status != CPC_OK:
        msg = load().cpc_last_error(ctx).decode(errors="replace")
        raise CpcError(status, msg)


def params_from_inp(p) -> cpc_params:
    """cpc_params from an InpParams (the .inp parameter set)."""
    c = cpc_params()
    c.which_corr, c.coordinates, c.estimator = p.which_corr, p.coordinates, p.estimator
    c.periodic_box, c.data_sorted, c.do_jk = int(p.periodic_box), p.data_sorted, p.do_jk
    c.n_jk = p.n_jk_regions
    c.sig_crit, c.rand_subsample = p.sig_crit, int(p.rand_subsample)
    c.n_bins, c.lin_bin, c.n_p_bin = p.n_bins, int(p.lin_bin), p.n_p_bin
    c.bin_r_min, c.bin_r_max = p.bin_r_min, p.bin_r_max
    c.p_min, c.p_max = p.p_min, p.p_max
    c.periodic_box_size = p.periodic_box_size
    c.z_max, c.dz, c.z_sep_max = p.z_max, p.dz, p.z_sep_max
    return c


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One GPU context (the state corels2 works on for one .inp parameter set).

    Sky runs (coordinates 0) also take the distance table (``table`` with
    columns z, H, DA, DC as data_ini reads them): the library needs H(z) and
    the transverse distance for the per-row windows, and z_sep_max is derived
    from the table as data_ini does."""

    def __init__(self, inp_params, table=None):
        self.lib = load()
        self.params = inp_params
        self._cp = params_from_inp(inp_params)
        self._table = None
        if inp_params.coordinates == 0:
            if table is None:
                raise ValueError("sky contexts need the distance table")
            from . import synth
            H = np.ascontiguousarray(table.H, dtype=np.float64)
            dA = np.ascontiguousarray(table.transverse if inp_params.use_comoving else table.DA,
                                      dtype=np.float64)
            self._table = (H, dA)
            self._cp.H_z, self._cp.dA_z, self._cp.n_table = H.ctypes.data, dA.ctypes.data, H.shape[0]
            self._cp.z_sep_max = synth.derived_z_sep(inp_params, table)[0]
        h = ctypes.c_void_p()
        check(self.lib.cpc_create(ctypes.byref(h), ctypes.byref(self._cp)))
        self.h = h
        nh, nb, npb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(self.lib.cpc_accum_shape(self.h, ctypes.byref(nh), ctypes.byref(nb),
                                       ctypes.byref(npb)), self.h)
        self.shape = (nh.value, nb.value, npb.value)
        self.sizes = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning(self, cells_per_rmax=0, pi_window=0, tile=0):
        check(self.lib.cpc_set_tuning(self.h, cells_per_rmax, pi_window, tile), self.h)

    def autotune(self, kind: str, slot_g1: int, slot_g2: int, sample_stride: int = 8):
        """Pick the fastest cell width and Pi window for this pair type on every
        sample_stride-th work unit; returns (cells_per_rmax, pi_window)."""
        k, w = ctypes.c_int(), ctypes.c_int()
        check(self.lib.cpc_autotune(self.h, PAIR[kind], slot_g1, slot_g2, sample_stride,
                                    ctypes.byref(k), ctypes.byref(w)), self.h)
        return k.value, w.value

    def upload(self, slot: int, cat) -> None:
        """cat: object with x, y, z and optional w, e1, e2, phi, jk, jk_prob, e3
        (kappa as e1 for which_corr 3, 4; the ED orientation as e1, e2, e3 for
        which_corr 5; dc, da for sky catalogues)."""
        keep = []

        def ptr(a, dt=np.float64):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data

        c = cpc_catalog()
        c.n = int(np.asarray(cat.x).shape[0])
        c.x, c.y, c.z = ptr(cat.x), ptr(cat.y), ptr(cat.z)
        c.w = ptr(getattr(cat, "w", None))
        c.e1, c.e2 = ptr(getattr(cat, "e1", None)), ptr(getattr(cat, "e2", None))
        c.phi = ptr(getattr(cat, "phi", None))
        c.jk = ptr(getattr(cat, "jk", None), np.int32)
        c.jk_prob = ptr(getattr(cat, "jk_prob", None))
        c.dc, c.da = ptr(getattr(cat, "dc", None)), ptr(getattr(cat, "da", None))
        c.e3 = ptr(getattr(cat, "e3", None))
        check(self.lib.cpc_upload(self.h, slot, ctypes.byref(c)), self.h)
        self.sizes[slot] = c.n

    def launches(self) -> int:
        v = ctypes.c_int64()
        check(self.lib.cpc_launch_count(self.h, ctypes.byref(v)), self.h)
        return v.value

    def set_shard(self, shard: int, n_shards: int) -> None:
        """Count only the work units i with i % n_shards == shard (fast box
        engine); the shards' raw blocks sum to the whole count."""
        check(self.lib.cpc_set_shard(self.h, shard, n_shards), self.h)

    def set_graph_replay(self, enable: bool) -> None:
        """Replay fast counts from a captured CUDA graph (default) or launch
        their kernels directly."""
        check(self.lib.cpc_set_graph_replay(self.h, 1 if enable else 0), self.h)

    def set_twin(self, enable: bool) -> None:
        """Twin counts on (default) or off: a cross term of two slots holding
        the same galaxies tests each unordered pair once and adds both orders."""
        check(self.lib.cpc_set_twin(self.h, 1 if enable else 0), self.h)

    def last_twin(self) -> bool:
        """Whether this context's last fast count ran as a twin count."""
        v = ctypes.c_int()
        check(self.lib.cpc_last_twin(self.h, ctypes.byref(v)), self.h)
        return bool(v.value)

    def graph_stats(self) -> tuple:
        """(captures, replays) of this context's fast-count graph."""
        c, r = ctypes.c_int64(), ctypes.c_int64()
        check(self.lib.cpc_graph_stats(self.h, ctypes.byref(c), ctypes.byref(r)), self.h)
        return c.value, r.value

    def new_accum(self):
        nh, nb, npb = self.shape
        num = np.zeros((nh, nb, npb), dtype=np.int64)
        sums = np.zeros((nh, nb, npb, NF), dtype=np.float64)
        acc = cpc_accum()
        acc.num, acc.sums = num.ctypes.data, sums.ctypes.data
        return acc, num, sums

    def count(self, kind: str, slot_g1: int, slot_g2: int, engine: str = "fast",
              row_stride: int = 1, row_offset: int = 0) -> dict:
        """One corels2 call: RAW region sums (h=0 full, h=1+r region r)."""
        acc, num, sums = self.new_accum()
        check(self.lib.cpc_count(self.h, PAIR[kind], slot_g1, slot_g2, ENGINE[engine],
                                 row_stride, row_offset, ctypes.byref(acc)), self.h)
        return {"num": num, "sums": sums, "n_window": acc.n_window, "n_binned": acc.n_binned,
                "n_rechecked": acc.n_rechecked, "kernel_ms": acc.kernel_ms,
                "pair_kernel_ms": acc.pair_kernel_ms}


    def count_async(self, kind: str, slot_g1: int, slot_g2: int, engine: str = "fast",
                    stream: int = 0, row_stride: int = 1, row_offset: int = 0) -> None:
        """Enqueue a count after the work on CUDA stream `stream` (a raw
        cudaStream_t handle, 0 = default stream); collect it with finish()."""
        check(self.lib.cpc_count_async(self.h, PAIR[kind], slot_g1, slot_g2, ENGINE[engine],
                                       row_stride, row_offset, ctypes.c_void_p(stream or None)),
              self.h)

    def finish(self) -> dict:
        """Wait for the count enqueued by count_async and return it like count()."""
        acc, num, sums = self.new_accum()
        check(self.lib.cpc_count_finish(self.h, ctypes.byref(acc)), self.h)
        return {"num": num, "sums": sums, "n_window": acc.n_window, "n_binned": acc.n_binned,
                "n_rechecked": acc.n_rechecked, "kernel_ms": acc.kernel_ms,
                "pair_kernel_ms": acc.pair_kernel_ms}

    def count_auto(self, kind: str, slot: int, engine: str = "fast", row_stride: int = 1,
                   row_offset: int = 0) -> dict:
        """One corels1 call (auto pairs of the catalogue in `slot`), kind "SS"
        or "RsRs": RAW region sums like count()."""
        acc, num, sums = self.new_accum()
        check(self.lib.cpc_count_auto(self.h, PAIR[kind], slot, ENGINE[engine], row_stride,
                                      row_offset, ctypes.byref(acc)), self.h)
        return {"num": num, "sums": sums, "n_window": acc.n_window, "n_binned": acc.n_binned,
                "n_rechecked": acc.n_rechecked, "kernel_ms": acc.kernel_ms,
                "pair_kernel_ms": acc.pair_kernel_ms}


def autotune_batch(jobs, sample_stride: int = 0) -> tuple:
    """jobs: list of (Context, kind, slot_g1, slot_g2) as for count_batch.
    Times batched launches on every sample_stride-th work unit of every job
    for the cell widths and Pi windows the single-job autotuner tries, keeps
    the fastest on every context and returns (cells_per_rmax, pi_window).
    sample_stride 0: the largest job's g1 rows // 25,000."""
    lib = load()
    n = len(jobs)
    if sample_stride <= 0:
        rows = max(j[0].sizes.get(j[2], 1) for j in jobs)
        sample_stride = max(1, rows // 25000)
    ctxs = (ctypes.c_void_p * n)(*[j[0].h.value for j in jobs])
    kinds = (ctypes.c_int * n)(*[PAIR[j[1]] for j in jobs])
    s1 = (ctypes.c_int * n)(*[j[2] for j in jobs])
    s2 = (ctypes.c_int * n)(*[j[3] for j in jobs])
    k, w = ctypes.c_int(), ctypes.c_int()
    check(lib.cpc_autotune_batch(n, ctxs, kinds, s1, s2, sample_stride, ctypes.byref(k),
                                 ctypes.byref(w)))
    return k.value, w.value


def count_batch(jobs) -> list:
    """jobs: list of (Context, kind, slot_g1, slot_g2); one persistent launch."""
    lib = load()
    n = len(jobs)
    ctxs = (ctypes.c_void_p * n)(*[j[0].h.value for j in jobs])
    kinds = (ctypes.c_int * n)(*[PAIR[j[1]] for j in jobs])
    s1 = (ctypes.c_int * n)(*[j[2] for j in jobs])
    s2 = (ctypes.c_int * n)(*[j[3] for j in jobs])
    accs = (cpc_accum * n)()
    keep = []
    for k, j in enumerate(jobs):
        a, num, sums = j[0].new_accum()
        accs[k] = a
        keep.append((num, sums))
    check(lib.cpc_count_batch(n, ctxs, kinds, s1, s2, accs))
    return [{"num": keep[k][0], "sums": keep[k][1], "n_window": accs[k].n_window,
             "n_binned": accs[k].n_binned, "n_rechecked": accs[k].n_rechecked,
             "kernel_ms": accs[k].kernel_ms,
             "pair_kernel_ms": accs[k].pair_kernel_ms} for k in range(n)]


def rand_uniform(seed: int, skip: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float64)
    check(load().cpc_host_rand_uniform(seed, skip, n, out.ctypes.data))
    return out


def elip_angle(e1, e2) -> np.ndarray:
    e1, e2 = _f64(e1), _f64(e2)
    out = np.empty_like(e1)
    check(load().cpc_host_elip_angle(e1.shape[0], e1.ctypes.data, e2.ctypes.data,
                                     out.ctypes.data))
    return out


def rp_thresholds(inp_params) -> np.ndarray:
    cp = params_from_inp(inp_params)
    out = np.empty(inp_params.n_bins + 1, dtype=np.float64)
    check(load().cpc_host_rp_thresholds(ctypes.byref(cp), out.ctypes.data))
    return out


def pi_thresholds(inp_params) -> np.ndarray:
    cp = params_from_inp(inp_params)
    out = np.empty(inp_params.n_p_bin + 1, dtype=np.float64)
    check(load().cpc_host_pi_thresholds(ctypes.byref(cp), out.ctypes.data))
    return out


def finalize_cross(inp_path: str, terms: dict, weights) -> None:
    """Finalisation + output files from RAW histogram blocks.  terms: dict with
    keys among SD, SRd, DRs, RsRd -> (num, sums); weights: 8 totals."""
    args = []
    for k in ("SD", "SRd", "DRs", "RsRd"):
        if k in terms:
            n, s = terms[k]
            n = np.ascontiguousarray(n, dtype=np.int64)
            s = np.ascontiguousarray(s, dtype=np.float64)
            terms[k] = (n, s)
            args += [n.ctypes.data, s.ctypes.data]
        else:
            args += [None, None]
    w = np.ascontiguousarray(weights, dtype=np.float64)
    check(load().cpc_host_finalize_cross(inp_path.encode(), *args, w.ctypes.data))


def finalize_auto(inp_path: str, terms: dict, weights) -> None:
    """Auto-correlation finalisation + output files from RAW blocks.  terms: keys
    among SS, SRs, RsRs -> (num, sums); weights: 8 totals (S and Rs used)."""
    args = []
    for k in ("SS", "SRs", "RsRs"):
        if k in terms:
            n, s = terms[k]
            n = np.ascontiguousarray(n, dtype=np.int64)
            s = np.ascontiguousarray(s, dtype=np.float64)
            terms[k] = (n, s)
            args += [n.ctypes.data, s.ctypes.data]
        else:
            args += [None, None]
    w = np.ascontiguousarray(weights, dtype=np.float64)
    check(load().cpc_host_finalize_auto(inp_path.encode(), *args, w.ctypes.data))


def count_fp64_noalloc(inp_params, kind: str, g1: dict, g2: dict, d_num: int, d_sums: int,
                       stream: int = 0) -> dict:
    """cpc_count_fp64_noalloc: g1/g2 map field name -> (device pointer or None)
    plus "n"; d_num/d_sums are device pointers to the output blocks."""
    lib = load()
    cp = params_from_inp(inp_params)

    def dc(g):
        c = cpc_device_catalog()
        c.n = int(g["n"])
        for f in ("x", "y", "z", "w", "e1", "e2", "phi", "jk", "jk_prob"):
            setattr(c, f, g.get(f))
        return c

    c1, c2 = dc(g1), dc(g2)
    nw, nb = ctypes.c_int64(), ctypes.c_int64()
    err = ctypes.create_string_buffer(512)
    st = lib.cpc_count_fp64_noalloc(ctypes.byref(cp), PAIR[kind], ctypes.byref(c1),
                                    ctypes.byref(c2), d_num, d_sums, ctypes.byref(nw),
                                    ctypes.byref(nb), stream or None, err, 512)
    if st != CPC_OK:
        raise CpcError(st, err.value.decode(errors="replace"))
    return {"n_window": nw.value, "n_binned": nb.value}
