"""The oracle (C restatement of corels2) pinned against the reference's own
outputs: golden fixtures generated by running the reference (tests/golden)."""
import numpy as np
import pytest

import oracle
import copy

from corr_pc_gb300 import synth
from helpers import AutoGolden, Golden, SkyGolden, auto_golden_names, golden_names, sky_golden_names


@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference(name):
    g = Golden(name)
    p = g.params
    cats = oracle.read_like_reference(p, [("S", g.S), ("D", g.D)])
    num, sums, n_total, n_in = oracle.port_corels2(p, "SD", cats["D"], cats["S"], n_threads=2)
    assert n_in == g.n_in
    assert n_total == g.n_total
    assert np.array_equal(num, g.raw_num)
    scale = np.abs(g.raw_sums).max(axis=(0, 1, 2)) + 1e-300
    assert (np.abs(sums - g.raw_sums) / scale).max() < 1e-12


def test_port_thread_count_independent():
    g = Golden("box_wgp_clustered")
    cats = oracle.read_like_reference(g.params, [("S", g.S), ("D", g.D)])
    a = oracle.port_corels2(g.params, "SD", cats["D"], cats["S"], n_threads=1)
    b = oracle.port_corels2(g.params, "SD", cats["D"], cats["S"], n_threads=4)
    assert np.array_equal(a[0], b[0]) and a[2:] == b[2:]
    assert np.allclose(a[1], b[1], rtol=1e-12, atol=1e-12)


def test_port_row_subsample_partitions():
    """Row subsamples with offsets 0..k-1 add up to the full count."""
    g = Golden("box_wgg_uniform")
    cats = oracle.read_like_reference(g.params, [("S", g.S), ("D", g.D)])
    full = oracle.port_corels2(g.params, "SD", cats["D"], cats["S"])
    parts = [oracle.port_corels2(g.params, "SD", cats["D"], cats["S"], row_stride=3, row_offset=o)
             for o in range(3)]
    assert np.array_equal(sum(q[0] for q in parts), full[0])
    assert sum(q[3] for q in parts) == full[3]


def test_glibc_rand_restatement():
    """The rand() restatement equals glibc's own stream (where glibc is the libc)."""
    import ctypes
    try:
        libc = ctypes.CDLL("libc.so.6")
    except OSError:
        pytest.skip("no glibc")
    libc.srand(124693517)
    ref = np.array([libc.rand() for _ in range(2000)], dtype=np.int32)
    assert np.array_equal(oracle.glibc_rand(124693517, 0, 2000), ref)
    assert np.array_equal(oracle.glibc_rand(124693517, 777, 100), ref[777:877])


@pytest.mark.parametrize("name", sky_golden_names())
def test_port_matches_reference_sky(name):
    """Sky terms SRd, RsRd, SD, DRs: windows (sky_calcs.cpp:105-196), great-circle
    r_p with the C library's trigonometry, comoving Pi, jackknife to both
    regions, table lookups of DC/DA."""
    g = SkyGolden(name)
    p = g.params
    cats = oracle.read_like_reference(p, g.read_order(), table=g.table)
    zsep = synth.derived_z_sep(p, g.table)[0]
    for t in g.terms:
        kind, a, b = SkyGolden.KIND[t]
        pp = p
        if t == "DRs" and g.meta["drs_as_wgg"]:
            pp = copy.copy(p)
            pp.which_corr = 0
        num, sums, n_total, n_in = oracle.port_corels2(pp, kind, cats[a], cats[b], n_threads=2,
                                                       H_z=g.table.H, dA_z=g.table.transverse,
                                                       z_sep_max=zsep)
        rnum, rsums, rin, rtot = g.term(t)
        assert (n_in, n_total) == (rin, rtot), t
        assert np.array_equal(num, rnum), t
        scale = np.abs(rsums).max(axis=(0, 1, 2)) + 1e-300
        assert (np.abs(sums - rsums) / scale).max() < 1e-12, t


@pytest.mark.parametrize("name", auto_golden_names())
def test_port_corels1_matches_reference(name):
    """corels1 (one catalogue, each pair once by index order, the +1 z image
    from row 0 when sorted) and the auto run's other terms."""
    g = AutoGolden(name)
    p = g.params
    cats = oracle.read_like_reference(p, g.read_order(), table=g.table)
    kw = {}
    if g.table is not None:
        kw = dict(H_z=g.table.H, dA_z=g.table.transverse,
                  z_sep_max=synth.derived_z_sep(p, g.table)[0])
    for t in g.terms:
        if t == "SS":
            res = oracle.port_corels1(p, "SS", cats["S"], n_threads=2, **kw)
        elif t == "RsRs":
            res = oracle.port_corels1(p, "RsRs", cats["Rs"], n_threads=2, **kw)
        elif t == "SRs":
            res = oracle.port_corels2(p, "SRs", cats["Rs"], cats["S"], n_threads=2, **kw)
        else:
            raise AssertionError(t)
        num, sums, n_total, n_in = res
        rnum, rsums, rin, rtot = g.term(t)
        assert (n_in, n_total) == (rin, rtot), t
        assert np.array_equal(num, rnum), t
        scale = np.abs(rsums).max(axis=(0, 1, 2)) + 1e-300
        assert (np.abs(sums - rsums) / scale).max() < 1e-12, t


def test_port_under_address_and_ub_sanitizers(tmp_path):
    """The C restatement built with AddressSanitizer and UndefinedBehaviorSanitizer
    passes every other test of this file (box, sky and auto golden runs, thread
    counts, row samples) with no report."""
    import os
    import shutil
    import subprocess
    import sys
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    here = os.path.dirname(os.path.abspath(__file__))
    src = os.path.join(os.path.dirname(here), "oracle", "cpc_oracle.c")
    so = str(tmp_path / "libcpc_oracle_asan.so")
    r = subprocess.run(["gcc", "-O1", "-g", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-fopenmp",
                        "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE", src,
                        "-o", so, "-lm"], capture_output=True, text=True)
    libasan = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True,
                             text=True).stdout.strip()
    if r.returncode != 0 or not os.path.isabs(libasan):
        pytest.skip("sanitizer runtime not available")
    env = dict(os.environ, LD_PRELOAD=libasan, ASAN_OPTIONS="detect_leaks=0",
               UBSAN_OPTIONS="print_stacktrace=1", CPC_ORACLE_SO=so)
    r = subprocess.run([sys.executable, "-m", "pytest", os.path.join(here, "test_oracle.py"),
                        "-q", "-p", "no:cacheprovider", "-k", "not sanitizers"],
                       capture_output=True, text=True, env=env, timeout=900, cwd=here)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "runtime error" not in r.stdout + r.stderr
    assert "ERROR: AddressSanitizer" not in r.stdout + r.stderr
