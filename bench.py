#!/usr/bin/env python3
"""Benchmark of the pair-counting hot path: binned pairs/s.

Default workload: the 20,000,000-point Neyman-Scott periodic box with shapes
(wgg + wg+ + w++ from one which_corr 2 count, 125 jackknife cubes, 25 log r_p
x 50 Pi bins, float32 positions) -- the configuration the headline target is
stated on.  Other workloads: --workload box_ns_wgp_200k | box_uniform_wgg_20k |
box_ns_wpp_2M (the 20M box's geometry at a tenth of the points: the profiling
case) | box_batch_wpp_64 | box_ns_ed_rmu_200k | box_ns_kappa_200k (the 200k
box with the ED and kappa variants) | sky_wgp_500k_5M | sky_wgp_50k_500k (sky
survey: SRd, RsRd, SD, DRs on a row sample).

One step = one corels2 call (the SD pair type these runs use).  On the 20M box
a step counts one of 20 shards of the work queue (the units i with
i % 20 == k % 20: every g2 candidate, a twentieth of the outer tiles), so 20
steps are one full count and the timed region stays near a minute; on the
other box workloads a step is the whole count.  `value` times the device work
with the catalogues resident in HBM (CUDA events on the library's stream around
the zeroing, the pair kernel and the FP64 edge recheck; the on-device cell-list
build is reported beside it as `cell_list`); the 20M box's inputs (2.3 GB per
catalogue) exceed L2, the smaller boxes flush L2 (256 MB write) between timed
steps.  `e2e` times the public C ABI from host buffers, wall clock: both
uploads (copy + on-device cell list) + the count + the histogram readback (one
full count on the 20M box).

`--impl reference` times the CPU implementation of the path on this host's
cores (the oracle restatement of corels2, fed as the reference's read path
feeds it; the reference binary itself is built from its sources only where
they exist and cannot travel to this host) on a bounded row sample per step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "binned pairs/s (wgg+wg+ w/ jackknife) vs plain FP64 GPU & host CPU; % roofline"
UNIT = "pairs/s"
DEFAULT_WORKLOAD = "box_ns_wpp_20M"
# work-queue shards of one full count (one shard per step)
SHARDS = {"box_ns_wpp_20M": 20}


def _workload(name: str):
    from corr_pc_gb300 import synth
    if name == "box_ns_wgp_200k":
        return [synth.box_ns_wgp()]
    if name == "box_uniform_wgg_20k":
        return [synth.box_uniform_wgg()]
    if name == "box_ns_wpp_20M":
        return [synth.box_ns_large_wpp()]
    if name == "box_ns_wpp_2M":
        # the 20M box's geometry and binning at a tenth of the parents: the
        # profiling case of the w++ kernel (one count about half a second)
        wl = synth.box_ns_large_wpp(n_parents=20000)
        wl.name = "box_ns_wpp_2M"
        return [wl]
    if name == "box_batch_wpp_64":
        return synth.box_batch_wpp()
    if name == "box_ns_ed_rmu_200k":
        return [synth.box_ns_ed_rmu()]
    if name == "box_ns_kappa_200k":
        return [synth.box_ns_kappa()]
    raise SystemExit(f"unknown workload {name}")


def _describe(wls) -> dict:
    p = wls[0].params
    name = wls[0].name if len(wls) == 1 else "box_batch_wpp_64"
    n_pts = int(sum(w.shape.n for w in wls))
    d = {"workload": name,
         "which_corr": p.which_corr, "coordinates": p.coordinates, "n_jk": p.n_jk_regions,
         "rp_bins": p.n_bins, "pi_bins": p.n_p_bin, "rp_range": [p.bin_r_min, p.bin_r_max],
         "pi_range": [p.p_min, p.p_max], "box": p.periodic_box_size,
         "n_points": n_pts, "n_catalogs": len(wls),
         "pair_type": "SD (shape x density, S and D the same points)",
         "l2": ("inputs larger than L2 (about 2.3 GB per uploaded catalogue)"
                if n_pts >= 10_000_000 else "flushed between timed steps (256 MB write)")}
    return d


def _step_definition(name: str, impl: str) -> str:
    if impl == "reference":
        return ("every k-th outer row of the corels2 call (offset changes every step), k sized "
                "for a bounded sample")
    k = SHARDS.get(name, 1)
    if k > 1:
        return (f"one corels2 call over one of {k} shards of the work queue (units i with "
                f"i % {k} == step % {k}); {k} steps = one full count")
    return "one corels2 call over the whole workload"


class ClockSampler:
    """nvidia-smi clocks during the timed region (read-only query)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int = 0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _profile_value(workload: str, key: str):
    """A figure of the committed ncu summary of the fast kernel on this workload
    (a table row "| key | value |")."""
    path = os.path.join(ROOT, "profiles", f"fast_pairs_kernel_{workload}.md")
    try:
        for line in open(path):
            if line.startswith(f"| {key} |"):
                return float(line.split("|")[2])
    except (OSError, ValueError):
        pass
    return None


def _profile_traffic(workload: str):
    """DRAM bytes per launch of the fast kernel (dram__bytes_read.sum +
    dram__bytes_write.sum) from the committed ncu summary of this workload."""
    return _profile_value(workload, "traffic_bytes_per_launch")


def _hbm_peak():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        return None


def _peaks() -> dict:
    """Live FP32 FFMA and shared-memory 32-bit atomic peaks (this GPU): the
    conflict-free reduction without a returned value, the kind the pair kernels
    issue."""
    from corr_pc_gb300 import build as b
    lib = ctypes.CDLL(b.PEAKS)
    lib.cpc_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                             ctypes.POINTER(ctypes.c_double)]
    out = {}
    for k, nm in ((0, "ffma_flops"), (1, "smem_atomic_u32_ops")):
        v = ctypes.c_double()
        rc = lib.cpc_peak(k, ctypes.byref(v), None)
        out[nm] = v.value if rc == 0 else None
    return out


def _oracle_cats(p, wl):
    """The oracle's inputs, derived from the synthetic catalogue the way the
    reference's read path derives them (glibc rand() jackknife draws in read
    order, elip_angle) by the oracle itself -- independent of the product
    library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the CPU baseline and checker (test infrastructure)
    return oracle.read_like_reference(p, [("S", wl.shape), ("D", wl.density)])


def _cpu_sample(p, ocats, budget_s: float, n_binned_full: int, threads: int, offset: int = 0):
    """Time the oracle restatement of corels2 on every k-th outer row."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the CPU baseline (test infrastructure)
    rate_guess = 4e6 * threads  # binned pairs/s on one ARM/x86 core, rough
    stride = max(1, int(n_binned_full / (rate_guess * budget_s)))
    t = time.perf_counter()
    num, sums, ntot, nin = oracle.port_corels2(p, "SD", ocats["D"], ocats["S"],
                                               n_threads=threads, row_stride=stride,
                                               row_offset=offset % stride)
    dt = time.perf_counter() - t
    return {"value": nin / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"every {stride}-th outer row (offset {offset % stride}): "
                      f"{nin} binned pairs in {dt:.2f} s"}, stride, nin, dt, (num, sums)


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wls = _workload(args.workload)
    wl = wls[0]
    p = wl.params
    ocats = _oracle_cats(p, wl)
    threads = os.cpu_count() or 1
    # estimate the full binned count cheaply from a tiny sample
    probe, stride0, nin0, _, _ = _cpu_sample(p, ocats, 0.5, 10 ** 12, threads)
    n_full = nin0 * stride0
    tot_pairs, tot_t, last = 0, 0.0, None
    for s in range(args.warmup + args.steps):
        res, stride, nin, dt, _ = _cpu_sample(p, ocats, args.ref_budget, n_full, threads,
                                              offset=s)
        if s >= args.warmup:
            tot_pairs += nin
            tot_t += dt
            last = res
    v = tot_pairs / tot_t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, in memory)", "config": _describe(wls),
            "step_definition": _step_definition(_describe(wls)["workload"], "reference"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": last["sample"] if last else ""},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# sky survey workload (coordinates 0): terms SRd, RsRd, SD, DRs
# ---------------------------------------------------------------------------

SKY_TERMS = (("SRd", "Rd", "S"), ("RsRd", "Rd", "Rs"), ("SD", "D", "S"), ("DRs", "Rs", "D"))
# row shards of one full pass over the four terms (one shard per step)
SKY_SHARDS = {"sky_wgp_500k_5M": 40, "sky_wgp_50k_500k": 4}
SKY_SLOTS = {"S": 0, "Rs": 1, "D": 2, "Rd": 3}


def _sky_setup(name):
    from corr_pc_gb300 import host, synth
    sizes = {"sky_wgp_500k_5M": (500000, 5000000), "sky_wgp_50k_500k": (50000, 500000)}
    if name not in sizes:
        raise SystemExit(f"unknown workload {name}")
    wl = synth.sky_wgp(*sizes[name])
    wl.name = name
    order = [("S", wl.shape), ("Rs", wl.shape_rand), ("D", wl.density), ("Rd", wl.density_rand)]
    cats = host.prepare(wl.params, order, table=wl.table)
    return wl, order, cats


def _sky_describe(wl, rows):
    p = wl.params
    return {"workload": wl.name, "which_corr": p.which_corr, "n_jk": p.n_jk_regions,
            "rp_bins": p.n_bins, "pi_bins": p.n_p_bin, "rp_range": [p.bin_r_min, p.bin_r_max],
            "pi_range": [p.p_min, p.p_max], "n_data": wl.shape.n, "n_randoms": wl.shape_rand.n,
            "patch_deg": [10, 10], "chi_range": [500, 1500],
            "pair_types": [t for t, _, _ in SKY_TERMS],
            "l2": "inputs larger than L2 (about 1.2 GB per random catalogue); L2 flushed "
                  "between steps"}


def _sky_strides(cats, rows):
    out = []
    for t, a, b in SKY_TERMS:
        n1 = max(cats[a].n, cats[b].n)
        out.append(max(1, n1 // rows))
    return out


def _sky_oracle_sample(wl, cats, budget_s, rows_hint, threads, offset=0):
    """The oracle restatement of corels2 on a row sample of every sky term."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the CPU baseline (test infrastructure)
    from corr_pc_gb300 import synth
    p = wl.params
    ocats = oracle.read_like_reference(p, [(r, c) for r, c in
                                           (("S", wl.shape), ("Rs", wl.shape_rand),
                                            ("D", wl.density), ("Rd", wl.density_rand))],
                                       table=wl.table)
    zsep = synth.derived_z_sep(p, wl.table)[0]
    strides = _sky_strides(cats, rows_hint)
    tot, dt = 0, 0.0
    hists = {}
    for (t, a, b), st in zip(SKY_TERMS, strides):
        t0 = time.perf_counter()
        num, sums, _, nin = oracle.port_corels2(p, t, ocats[a], ocats[b], n_threads=threads,
                                                row_stride=st, row_offset=offset % st,
                                                H_z=wl.table.H, dA_z=wl.table.transverse,
                                                z_sep_max=zsep)
        dt += time.perf_counter() - t0
        tot += nin
        hists[t] = (num, sums, st, offset % st)
        if dt > budget_s:
            break
    return tot, dt, hists


def run_sky(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl, order, cats = _sky_setup(args.workload)
    threads = os.cpu_count() or 1
    if args.impl == "reference":
        tot_pairs, tot_t = 0, 0.0
        rows = args.sky_cpu_rows
        for s in range(args.warmup + args.steps):
            n, dt, _ = _sky_oracle_sample(wl, cats, 1e9, rows, threads, offset=s)
            if s >= args.warmup:
                tot_pairs += n
                tot_t += dt
        v = tot_pairs / tot_t
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded, in memory)", "config": _sky_describe(wl, rows),
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": f"about {rows} outer rows per pair type per step"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from corr_pc_gb300 import build as b
    b.build()
    from corr_pc_gb300 import _lib, metrics
    p = wl.params
    ctx = _lib.Context(p, table=wl.table)
    for r, c in cats.items():
        ctx.upload(SKY_SLOTS[r], c)
    rows = args.sky_rows
    strides = _sky_strides(cats, rows)
    K = SKY_SHARDS.get(wl.name, 1)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    jobs = [(ctx, t, SKY_SLOTS[a], SKY_SLOTS[bb]) for t, a, bb in SKY_TERMS]

    def step(k):
        """Shard k % K of the four terms, in one launch of the fast kernel."""
        ctx.set_shard(k % K, K)
        rs = _lib.count_batch(jobs)
        return (sum(r["n_binned"] for r in rs), sum(r["n_window"] for r in rs),
                rs[0]["kernel_ms"])

    def step_rows(k, engine, mult=1):
        """Every st-th outer row of each term (the FP64 kernel's sample), one
        launch per term."""
        ctx.set_shard(0, 1)
        nb = nw = 0
        ms = 0.0
        for (t, a, bb), st in zip(SKY_TERMS, strides):
            st = st * mult
            r = ctx.count(t, SKY_SLOTS[a], SKY_SLOTS[bb], engine=engine, row_stride=st,
                          row_offset=k % st)
            nb += r["n_binned"]
            nw += r["n_window"]
            ms += r["kernel_ms"]
        return nb, nw, ms

    for k in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize()
        step(k)
    l0 = ctx.launches()
    n_bin = n_win = 0
    tot_ms = 0.0
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            nb, nw, ms = step(args.warmup + k)
            n_bin += nb
            n_win += nw
            tot_ms += ms
    launches = ctx.launches() - l0
    ctx.set_shard(0, 1)
    value = n_bin / (tot_ms * 1e-3)
    # end to end: the four uploads (host windows, device sort) + the four terms
    # over every outer row in one launch
    h2d = sum(8 * 9 * c.n + 4 * c.n + c.n for c in cats.values())
    t0 = time.perf_counter()
    for r, c in cats.items():
        ctx.upload(SKY_SLOTS[r], c)
    rs_e = _lib.count_batch(jobs)
    e2e_t = time.perf_counter() - t0
    nb_e = sum(r["n_binned"] for r in rs_e)
    nh, nbins, npb = ctx.shape
    d2h = 4 * nh * nbins * npb * (8 + 8 * _lib.NF)
    # plain FP64 sky kernel on an 8x sparser row sample
    nb64, _, ms64 = step_rows(0, "fp64", mult=8)
    fp64 = {"value": nb64 / (ms64 * 1e-3), "unit": UNIT,
            "sample": f"8x sparser row sample: {nb64} binned pairs in {ms64:.1f} ms"}
    fp64["speedup_of_fast"] = value / fp64["value"]
    cpu = None
    accuracy = None
    if not args.no_cpu:
        n, dt, hists = _sky_oracle_sample(wl, cats, args.cpu_budget, args.sky_cpu_rows, threads)
        cpu = {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"about {args.sky_cpu_rows} outer rows per pair type: {n} binned "
                         f"pairs in {dt:.2f} s"}
        # the fast kernel on the same rows of every term, against the oracle
        accuracy = {"against": "oracle (FP64 restatement of corels2) on the CPU-baseline rows",
                    "rows": cpu["sample"], "terms": {}}
        for (t, a, bb) in SKY_TERMS:
            if t not in hists:
                continue
            onum, osums, st, off = hists[t]
            rf = ctx.count(t, SKY_SLOTS[a], SKY_SLOTS[bb], row_stride=st, row_offset=off)
            accuracy["terms"][t] = metrics.accuracy_report(rf["num"], rf["sums"], onum, osums)
        accuracy["ok"] = all(v["ok"] for v in accuracy["terms"].values())
    peaks = _peaks()
    F = metrics.flops_per_pair(p.which_corr, p.coordinates)
    A = metrics.smem_updates_per_pair(p.which_corr, bool(p.do_jk))
    achieved_flops = F * value
    roofline = {"bound": "fp32", "achieved": achieved_flops / 1e12,
                "peak": (peaks["ffma_flops"] or float("nan")) / 1e12, "unit": "TFLOP/s",
                "frac": achieved_flops / peaks["ffma_flops"] if peaks["ffma_flops"] else None,
                "traffic": None, "kernel": "sky_warp_kernel",
                "kernel_ms_per_launch": tot_ms / args.steps,
                "work_per_pair": {"fp32_flops": F, "smem_atomic_updates": A},
                "peak_source": "measured live in this run (FFMA microbenchmark)"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded generator, in memory)", "config": _sky_describe(wl, rows),
            "step_definition": f"the four terms in one launch over one of {K} row shards "
                               f"(redshift-ordered positions k % {K} == step % {K}); {K} steps "
                               "= one full count of every term",
            "n_binned_per_step": n_bin / args.steps, "n_window_per_step": n_win / args.steps,
            "roofline": roofline, "cpu_baseline": cpu, "fp64_gpu": fp64, "accuracy": accuracy,
            "e2e": {"value": nb_e / e2e_t, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_t},
            "gpu_launches": launches, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD)
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU baseline")
    ap.add_argument("--ref-budget", type=float, default=5.0, help="seconds per reference step")
    ap.add_argument("--fp64-budget", type=float, default=3.0,
                    help="seconds of FP64 kernel (0: skip)")
    ap.add_argument("--cell-fp64-pairs", type=float, default=1e10,
                    help="binned pairs of the cell-list FP64 comparison (0: skip)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner")
    ap.add_argument("--tune", default=None,
                    help="K,W: fixed cell width r_max/K and Pi window W (instead of the autotuner)")
    ap.add_argument("--sky-rows", type=int, default=20000,
                    help="outer rows per pair type per step (sky workloads)")
    ap.add_argument("--sky-cpu-rows", type=int, default=400,
                    help="outer rows per pair type for the CPU baseline (sky workloads)")
    args = ap.parse_args()
    if args.workload.startswith("sky"):
        run_sky(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from corr_pc_gb300 import build as b
    b.build()
    from corr_pc_gb300 import _lib, host, metrics

    wls = _workload(args.workload)
    wl_name = _describe(wls)["workload"]
    n_shards = SHARDS.get(wl_name, 1)
    big = sum(w.shape.n for w in wls) >= 10_000_000  # inputs far larger than L2
    preps = [host.prepare(w.params, [("S", w.shape), ("D", w.density)]) for w in wls]
    ctxs = [_lib.Context(w.params) for w in wls]
    tuning = None
    if args.tune:
        tk, tw = (int(v) for v in args.tune.split(","))
        for c in ctxs:
            c.set_tuning(tk, tw)
        tuning = {"cells_per_rmax": tk, "pi_window": tw, "by": "--tune"}
    t_up = time.perf_counter()
    for c, cat in zip(ctxs, preps):
        c.upload(0, cat["D"])
        c.upload(1, cat["S"])
    torch.cuda.synchronize()
    upload_s = time.perf_counter() - t_up
    if len(ctxs) == 1 and not args.no_tune and not args.tune:  # outside the timed region
        n_rows = wls[0].density.n
        k, w = ctxs[0].autotune("SD", 0, 1, sample_stride=max(1, n_rows // 25000))
        tuning = {"cells_per_rmax": k, "pi_window": w if w else "automatic (every mu bin that fits)",
                  "by": "cpc_autotune on a shard of the work units"}
    elif len(ctxs) > 1 and not args.no_tune and not args.tune:
        k, w = _lib.autotune_batch([(c, "SD", 0, 1) for c in ctxs])
        tuning = {"cells_per_rmax": k, "pi_window": w,
                  "by": "cpc_autotune_batch on a shard of every box's work units"}
    # the uploads (copy, device checks, radix sort into the cell list, gather of
    # the SoA streams, host bucket tables), wall clock, outside the timed steps
    cell_list = {"upload_wall_ms_per_catalog": 1e3 * upload_s / (2 * len(ctxs)),
                 "catalogs": 2 * len(ctxs),
                 "note": "cpc_upload from host buffers: H2D copy, on-device checks, radix sort "
                         "by (column, region, z), gather of the SoA streams, bucket tables"}
    flush = None if big else torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def step(k=0, sharded=True):
        if len(ctxs) == 1:
            if n_shards > 1:
                if sharded:
                    ctxs[0].set_shard(k % n_shards, n_shards)
                else:
                    ctxs[0].set_shard(0, 1)
            r = ctxs[0].count("SD", 0, 1)
            return r["n_binned"], r["kernel_ms"], r["pair_kernel_ms"], r["n_window"]
        rs = _lib.count_batch([(c, "SD", 0, 1) for c in ctxs])
        return (sum(r["n_binned"] for r in rs), rs[0]["kernel_ms"], rs[0]["pair_kernel_ms"],
                sum(r["n_window"] for r in rs))

    for k in range(args.warmup):
        if flush is not None:
            flush.zero_()
        torch.cuda.synchronize()
        step(k)
    l0 = sum(c.launches() for c in ctxs)
    tot_ms = tot_pair_ms = 0.0
    n_bin = n_win = 0
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            if flush is not None:
                flush.zero_()
            torch.cuda.synchronize()
            nb, ms, pms, nw = step(args.warmup + k)
            n_bin += nb
            n_win += nw
            tot_ms += ms
            tot_pair_ms += pms
    torch.cuda.synchronize()
    launches = sum(c.launches() for c in ctxs) - l0
    twin_used = ctxs[0].last_twin()
    if n_shards > 1:
        ctxs[0].set_shard(0, 1)
    g_cap, g_rep = ctxs[0].graph_stats()
    t_step = tot_ms / args.steps
    if dist:
        tt = torch.tensor([t_step], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
        nn = torch.tensor([float(n_bin)], device="cuda")
        dist.all_reduce(nn)
        n_bin_all = float(nn.item())
    else:
        n_bin_all = float(n_bin)
    value = n_bin_all / args.steps / (t_step * 1e-3)

    # ---- end to end through the C ABI from host buffers ----
    h2d = 0
    for cat in preps:
        for g in (cat["D"], cat["S"]):
            h2d += 8 * 7 * g.n + 4 * g.n  # x y z w e1 e2 phi (f64), jk (i32); keep 1 B
            h2d += g.n
    d2h_hist = sum(c.shape[0] * c.shape[1] * c.shape[2] * (8 + 8 * _lib.NF) for c in ctxs)
    d2h = d2h_hist + sum(20 * (cat["D"].n + cat["S"].n) for cat in preps)
    # the 20M box: one full count (all shards); the others: up to 5 repeats
    e2e_steps = 1 if n_shards > 1 else max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    e2e_bin = 0
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for c, cat in zip(ctxs, preps):
            c.upload(0, cat["D"])
            c.upload(1, cat["S"])
        e2e_bin += step(sharded=False)[0]
    e2e_t = (time.perf_counter() - t0) / e2e_steps
    e2e_value = e2e_bin / e2e_steps / e2e_t
    if n_shards > 1:  # one full count: the value's timed steps together count it once
        full_pairs = e2e_bin / e2e_steps
    else:
        full_pairs = n_bin / args.steps

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    p = wls[0].params
    peaks = _peaks()
    F = metrics.flops_per_pair(p.which_corr, p.coordinates)
    A = metrics.smem_updates_per_pair(p.which_corr, bool(p.do_jk))
    pair_s = tot_pair_ms / args.steps * 1e-3
    n_per_step = n_bin / args.steps
    achieved_flops = F * n_per_step / pair_s
    achieved_atom = A * n_per_step / pair_s
    traffic = _profile_traffic(_describe(wls)["workload"])
    hbm_peak = _hbm_peak()
    hbm = None
    if traffic is not None:
        hbm_gbs = traffic / (tot_pair_ms / args.steps * 1e-3) / 1e9
        hbm = {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s",
               "frac": hbm_gbs / hbm_peak if hbm_peak else None,
               "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
               "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, "
                                 "profiles/fast_pairs_kernel_<workload>.md"}
    roofline = {"bound": "fp32", "achieved": achieved_flops / 1e12,
                "peak": (peaks["ffma_flops"] or float("nan")) / 1e12, "unit": "TFLOP/s",
                "frac": achieved_flops / peaks["ffma_flops"] if peaks["ffma_flops"] else None,
                "traffic": traffic,
                "kernel": "fast_pairs_kernel", "kernel_ms_per_launch": tot_pair_ms / args.steps,
                "work_per_pair": {"fp32_flops": F, "smem_atomic_updates": A},
                "peak_source": "measured live in this run (FFMA microbenchmark); "
                               "MEASURED_PEAKS.json has HBM and bf16 peaks only",
                "smem_atomics": {"achieved": achieved_atom / 1e12,
                                 "peak": (peaks["smem_atomic_u32_ops"] or float("nan")) / 1e12,
                                 "unit": "Tops/s",
                                 "frac": achieved_atom / peaks["smem_atomic_u32_ops"]
                                 if peaks["smem_atomic_u32_ops"] else None},
                "hbm": hbm}
    wl_name = _describe(wls)["workload"]
    pipe = _profile_value(wl_name, "shared_pipe_wavefronts_pct_of_peak")
    if pipe is not None:
        # the resource that binds the kernel, measured by ncu on this workload:
        # shared-memory wavefronts (histogram reductions scattered over the 32
        # banks, plus the staged-candidate and row loads) and instruction issue
        roofline["binding"] = {
            "resource": "shared-memory pipe (wavefronts) and instruction issue",
            "shared_pipe_frac": pipe / 100.0,
            "issue_active_frac": (_profile_value(wl_name, "issue_active_pct") or float("nan")) / 100.0,
            "wavefronts_per_binned_pair": _profile_value(wl_name, "shared_wavefronts_per_binned_pair"),
            "source": f"ncu --set full, profiles/fast_pairs_kernel_{wl_name}.md"}
    # plain FP64 GPU kernel on a bounded row sample of the same workload
    fp64 = None
    if len(ctxs) == 1 and args.fp64_budget > 0:
        # at least 4,000 outer rows: the plain kernel runs one thread per row, and
        # fewer rows leave the GPU idle (on the 20M box 1,000 rows give 1.2e7
        # pairs/s, 4,000 2.2e7, 16,000 2.7e7)
        est_rate = 1.5e8 if not big else 2e7
        n_rows = wls[0].density.n
        stride = max(1, min(int(full_pairs / (est_rate * args.fp64_budget)), n_rows // 4000))
        r64 = ctxs[0].count("SD", 0, 1, engine="fp64", row_stride=stride)
        fp64 = {"value": r64["n_binned"] / (r64["kernel_ms"] * 1e-3), "unit": UNIT,
                "sample": f"every {stride}-th outer row: {r64['n_binned']} binned pairs in "
                          f"{r64['kernel_ms']:.1f} ms"}
        fp64["speedup_of_fast"] = value / fp64["value"]
    # the same cell list and work units with every window candidate evaluated by
    # the FP64 path (the reference's double arithmetic, global atomics): the
    # precision comparison at equal algorithm, on one shard of the work queue
    # sized for about args.cell_fp64_pairs binned pairs, against the fast engine
    # on the same shard counting every order (a twin count's shard holds other
    # pairs: both orders of the pairs whose row it holds)
    cell64 = None
    if len(ctxs) == 1 and args.cell_fp64_pairs > 0:
        K = max(1, int(full_pairs / args.cell_fp64_pairs))
        ctxs[0].set_shard(0, K)
        rc = ctxs[0].count("SD", 0, 1, engine="cell_fp64")
        ctxs[0].set_twin(False)
        rfs = ctxs[0].count("SD", 0, 1)
        ctxs[0].set_twin(True)
        ctxs[0].set_shard(0, 1)
        v64 = rc["n_binned"] / (rc["kernel_ms"] * 1e-3)
        vf = rfs["n_binned"] / (rfs["kernel_ms"] * 1e-3)
        cell64 = {"value": v64, "unit": UNIT,
                  "sample": f"shard 0 of {K} of the work queue: {rc['n_binned']} binned pairs in "
                            f"{rc['kernel_ms']:.1f} ms",
                  "fast_on_same_shard": vf, "speedup_of_fast": vf / v64,
                  "speedup_of_value": value / v64,
                  "counts_equal_fast": bool(np.array_equal(rc["num"], rfs["num"])),
                  "accuracy_fast_vs_cell_fp64": metrics.accuracy_report(
                      rfs["num"], rfs["sums"], rc["num"], rc["sums"])["ok"]}
    cpu = None
    accuracy = None
    if not args.no_cpu and len(wls) == 1:
        ocats = _oracle_cats(p, wls[0])
        cpu, cstride, _, _, (onum, osums) = _cpu_sample(p, ocats, args.cpu_budget,
                                                        full_pairs, os.cpu_count() or 1)
        # the fast kernel on the same rows, checked against the oracle's FP64 histograms
        rf = ctxs[0].count("SD", 0, 1, row_stride=cstride)
        accuracy = dict(metrics.accuracy_report(rf["num"], rf["sums"], onum, osums),
                        against="oracle (FP64 restatement of corels2) on the CPU-baseline rows",
                        rows=cpu["sample"])
    elif fp64 is not None:
        rf = ctxs[0].count("SD", 0, 1, row_stride=stride)
        accuracy = dict(metrics.accuracy_report(rf["num"], rf["sums"], r64["num"], r64["sums"]),
                        against="plain FP64 GPU kernel on its rows", rows=fp64["sample"])
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64", "data": "synthetic (seeded generator, in memory)",
            "config": dict(_describe(wls), tuning=tuning,
                           pair_orders=("twin count: S and D hold the same galaxies, each "
                                        "unordered pair tested once and both orders added"
                                        if twin_used else "every order counted separately")),
            "step_definition": _step_definition(wl_name, "gb300"),
            "value_scope": "device time of the count (zeroing, pair kernel, FP64 edge recheck) "
                           "with both catalogues' cell lists resident; the cell-list build is "
                           "`cell_list`, everything from host buffers is `e2e`",
            "n_binned_per_step": n_per_step, "n_binned_full_count": full_pairs,
            "n_window_per_step": n_win / args.steps, "cell_list": cell_list,
            "roofline": roofline, "cpu_baseline": cpu, "fp64_gpu": fp64,
            "cell_list_fp64_gpu": cell64, "accuracy": accuracy,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_t},
            "gpu_launches": launches,
            "cuda_graph": {"captures": g_cap, "replays": g_rep,
                           "note": "each step replays the captured zeroing + pair kernel + "
                                   "recheck; captures include the autotuner's trial counts"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
