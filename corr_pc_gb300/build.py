"""Build the GB300 library in-tree (no cmake, no setuptools).

Produces ``corr_pc_gb300/_build/libcorrpc_gb300.so`` (CUDA kernels for
sm_103a + the C ABI of include/corrpc.h) and ``corr_pc_gb300/_build/corr_pc_gb300``
(the host driver: the reference's ``corr_pc`` command line on top of the ABI).
Translation units compile in parallel; up-to-date objects are reused.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libcorrpc_gb300.so")
CLI = os.path.join(OUT, "corr_pc_gb300")
PEAKS = os.path.join(OUT, "libcpc_peaks.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["cell_list.cu", "pair_fast.cu", "pair_fp64.cu", "pair_sky.cu", "capi.cu",
              "pair_noalloc.cu"]
CPP_SOURCES = ["host_helpers.cpp"]
HOST_SOURCES = ["host/inp.cpp", "host/reader.cpp", "host/finalize.cpp", "host/outp.cpp",
                "host/driver.cpp"]
HEADERS = ["cpc_device.cuh", "kernels.h", "host_helpers.h", "pair_values.h", "host/host.h",
           "df32.cuh", "pair_df.cuh", "param_check.h"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _stale(obj, deps):
    return not os.path.exists(obj) or os.path.getmtime(obj) < _newest(deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(os.path.join(OUT, "host"), exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "corrpc.h")]
    jobs = []
    objs = []
    nv = nvcc()
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-c", src, "-o", obj])
    for s in CPP_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OUT, s.replace(".cpp", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-c", src,
                         "-o", obj])
    host_objs = []
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, s)
        if not os.path.exists(src):
            continue
        obj = os.path.join(OUT, s.replace(".cpp", ".o"))
        host_objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC",
                         "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr, file=sys.stderr)
    lib_objs = objs + [o for o in host_objs if not o.endswith("driver.o")]
    if force or _stale(LIB, lib_objs):
        _run([nv, *ARCH, "-shared", "-o", LIB, *lib_objs, "-Xcompiler", "-fPIC"])
    psrc = os.path.join(CSRC, "peaks.cu")
    if force or _stale(PEAKS, [psrc]):
        _run([nv, *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", psrc, "-o", PEAKS])
    drv = [o for o in host_objs if o.endswith("driver.o")]
    if drv and (force or _stale(CLI, drv + [LIB])):
        _run(["g++", "-o", CLI, *drv, "-L" + OUT, "-lcorrpc_gb300",
              "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
