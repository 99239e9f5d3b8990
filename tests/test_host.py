"""Host side of the library (no GPU): exported ABI, read-path helpers,
bin thresholds, parameter files, finalisation against the reference's files."""
import math
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from corr_pc_gb300 import _lib, host, synth
from helpers import (AutoGolden, Golden, SkyGolden, auto_golden_names, compare_files,
                     golden_names, sky_golden_names)

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "corrpc.h")).read()
    declared = sorted(set(re.findall(r"\b(cpc_[a-z_0-9]+)\s*\(", hdr)))
    assert declared, "no declarations found"
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (cpc_[a-z_0-9]+)", out))
    missing = [d for d in declared if d not in exported]
    assert not missing, f"declared but not exported: {missing}"
    lib = _lib.load()
    for d in declared:
        assert hasattr(lib, d)
    assert lib.cpc_version().startswith(b"corr_pc_gb300")


def test_rand_stream_matches_oracle_and_glibc():
    r = _lib.rand_uniform(124693517, 0, 5000)
    o = oracle.glibc_rand(124693517, 0, 5000) / (2147483647 + 1.0)
    assert np.array_equal(r, o)
    assert np.array_equal(_lib.rand_uniform(124693517, 1234, 10), o[1234:1244])


def test_host_exception_becomes_a_status():
    """A C++ exception inside an entry point (here the length_error of a host
    vector longer than its max_size, thrown before anything is allocated) comes
    back as a status and a message instead of ending the process."""
    lib = _lib.load()
    out = np.empty(1)
    st = lib.cpc_host_rand_uniform(1, 0, 1 << 62, out.ctypes.data)
    assert _lib.STATUS_NAMES[st] == "CPC_ERR_NOMEM"
    assert b"host allocation too large" in lib.cpc_last_error(None)
    # the library keeps working afterwards
    assert np.array_equal(_lib.rand_uniform(7, 0, 3), oracle.glibc_rand(7, 0, 3) / 2147483648.0)


def test_context_free_messages_are_per_thread():
    """cpc_last_error(NULL) reports the calling thread's own last failure."""
    import threading
    lib = _lib.load()
    assert lib.cpc_host_rand_uniform(1, 0, -1, None) != 0
    seen = []

    def other():
        assert lib.cpc_host_rp_thresholds(None, None) != 0
        seen.append(lib.cpc_last_error(None))

    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert seen == [b"null argument"]
    assert lib.cpc_last_error(None) == b"bad arguments"


def test_status_codes_match_header():
    text = open(os.path.join(os.path.dirname(__file__), "..", "include", "corrpc.h")).read()
    enum = text[text.index("typedef enum {"):text.index("} cpc_status;")]
    codes = {int(v): k for k, v in re.findall(r"(CPC_\w+) = (\d+)", enum)}
    assert codes == _lib.STATUS_NAMES


def test_elip_angle_matches_reference_formula():
    rng = np.random.default_rng(3)
    e1, e2 = rng.normal(0, 0.5, 4000), rng.normal(0, 0.5, 4000)
    e1[:3] = [0.0, -0.0, 0.0]
    e2[:3] = [0.0, 0.3, -0.3]
    assert np.array_equal(_lib.elip_angle(e1, e2), oracle.elip_angle(e1, e2))


@pytest.mark.parametrize("lin", [0, 1])
def test_rp_thresholds_reproduce_reference_binning(lin):
    p = synth.box_ns_wgp().params
    p.lin_bin = lin
    thr = _lib.rp_thresholds(p)
    if lin:
        rs = (p.bin_r_max - p.bin_r_min) / p.n_bins
        f = lambda r: math.floor((r - p.bin_r_min) / rs)
    else:
        rs = (math.log10(p.bin_r_max) - math.log10(p.bin_r_min)) / p.n_bins
        f = lambda r: math.floor(math.log10(r / p.bin_r_min) / rs) if r > 0 else -10 ** 9
    for k in range(p.n_bins + 1):
        assert f(thr[k]) >= k
        assert f(np.nextafter(thr[k], 0.0)) < k
    rng = np.random.default_rng(0)
    for r in rng.uniform(0, p.bin_r_max * 1.1, 20000):
        want = f(r)
        got = int(np.searchsorted(thr, r, side="right")) - 1
        if 0 <= want < p.n_bins:
            assert got == want
        else:
            assert got < 0 or got >= p.n_bins


def test_pi_thresholds_reproduce_reference_binning():
    p = synth.box_uniform_wgg().params
    thr = _lib.pi_thresholds(p)
    ps = (p.p_max - p.p_min) / p.n_p_bin
    f = lambda x: math.floor((x - p.p_min) / ps)
    for k in range(p.n_p_bin + 1):
        assert f(thr[k]) >= k and f(np.nextafter(thr[k], -np.inf)) < k


def test_inp_round_trip(tmp_path):
    p = synth.box_ns_wgp().params
    p.out_file = str(tmp_path / "out_")
    path = str(tmp_path / "x.inp")
    p.write(path)
    q = synth.InpParams.read(path)
    for _k, a, _t in synth.INP_KEYS:
        assert getattr(p, a) == getattr(q, a), a


@pytest.mark.parametrize("name", ["box_wpp_weighted_distinct", "box_ed_rmu", "box_kappa_unsorted",
                                  "box_sk_distinct"])
def test_prepare_matches_reference_read_path(name):
    """The host read path (jackknife draws, phi, weights, and which samples carry
    e, kappa or the normalised ED orientation) equals the oracle's."""
    g = Golden(name)
    a = host.prepare(g.params, [("S", g.S), ("D", g.D)])
    b = oracle.read_like_reference(g.params, [("S", g.S), ("D", g.D)])
    for role in ("S", "D"):
        assert np.array_equal(a[role].jk_prob, b[role].jk_prob)
        assert np.array_equal(a[role].phi, b[role].phi)
        assert np.array_equal(a[role].w, b[role].w)
        for f in ("e1", "e2", "e3"):
            u, v = getattr(a[role], f), getattr(b[role], f)
            assert (u is None) == (v is None), (role, f)
            if u is not None:
                assert np.array_equal(u, v), (role, f)


def test_create_rejects_bad_parameters():
    p = synth.box_uniform_wgg().params
    p.n_bins = 0
    with pytest.raises(_lib.CpcError) as e:
        _lib.Context(p)
    assert e.value.status == 1
    p = synth.box_uniform_wgg().params
    p.sig_crit = 1
    with pytest.raises(_lib.CpcError):
        _lib.Context(p)
    p = synth.box_uniform_wgg().params
    p.coordinates = 3
    with pytest.raises(_lib.CpcError):
        _lib.Context(p)
    p = synth.box_uniform_wgg().params
    p.which_corr = 6
    with pytest.raises(_lib.CpcError):
        _lib.Context(p)
    p = synth.box_uniform_wgg().params
    p.coordinates, p.periodic_box = 7, 0  # r-mu outside a periodic box
    with pytest.raises(_lib.CpcError):
        _lib.Context(p)


@pytest.mark.parametrize("name", golden_names())
def test_finalisation_matches_reference_files(name, tmp_path):
    """Reference raw histograms -> this library's finalisation -> the
    reference's own output files."""
    g = Golden(name)
    p = g.params
    p.out_file = str(tmp_path) + "/run_"
    inp = str(tmp_path / "run.inp")
    p.write(inp)
    _lib.finalize_cross(inp, {"SD": (g.raw_num, g.raw_sums)}, g.weights())
    for fname, ref in g.files.items():
        got = open(p.out_file + fname).read()
        if fname.endswith(".info"):
            continue
        compare_files(got, ref, label=f"{name}:{fname}")


@pytest.mark.parametrize("name", sky_golden_names())
def test_sky_finalisation_matches_reference_files(name, tmp_path):
    """Reference raw histograms of the four sky terms -> Landy-Szalay
    finalisation -> the reference's own output files."""
    g = SkyGolden(name)
    p = g.params
    p.out_file = str(tmp_path) + "/run_"
    p.distance_file = str(tmp_path / "distances.dat")
    g.table.write(p.distance_file)
    inp = str(tmp_path / "run.inp")
    p.write(inp)
    terms = {t: g.term(t)[:2] for t in g.terms}
    w = []
    for role in ("S", "D", "Rs", "Rd"):
        c = g.cats[role]
        ww = np.ones(c.n) if c.w is None else c.w
        w += [float(ww.sum()), float((ww * ww).sum())]
    _lib.finalize_cross(inp, terms, w)
    for fname, ref in g.files.items():
        if fname.endswith(".info"):
            continue
        compare_files(open(p.out_file + fname).read(), ref, label=f"{name}:{fname}")


@pytest.mark.parametrize("name", auto_golden_names())
def test_auto_finalisation_matches_reference_files(name, tmp_path):
    """Reference raw histograms of an auto run (SS; SRs and RsRs on the sky) ->
    final_calc_auto (with re_bin for estimator 2) -> the reference's files."""
    g = AutoGolden(name)
    p = g.params
    p.out_file = str(tmp_path) + "/run_"
    if g.table is not None:
        p.distance_file = str(tmp_path / "distances.dat")
        g.table.write(p.distance_file)
    inp = str(tmp_path / "run.inp")
    p.write(inp)
    terms = {t: g.term(t)[:2] for t in g.terms}
    w = []
    for role in ("S", "S", "Rs", "Rs"):
        c = g.cats.get(role)
        if c is None:
            w += [0.0, 0.0]
            continue
        ww = np.ones(c.n) if c.w is None else c.w
        w += [float(ww.sum()), float((ww * ww).sum())]
    _lib.finalize_auto(inp, terms, w)
    assert g.files
    for fname, ref in g.files.items():
        if fname.endswith(".info"):
            continue
        compare_files(open(p.out_file + fname).read(), ref, label=f"{name}:{fname}")


def test_integration_binding_links_into_the_reference():
    """The corels2/corels1 binding (corr_pc_gb300/csrc/binding/corr_gpu.cpp)
    compiles against the reference's own headers and links, with the
    reference's objects (its pair loops renamed away) and main.cpp, into a
    corr_pc executable that calls this library.  It is built where the
    reference's sources are and not run (they do not exist on the GPU
    machines); test_gpu_cli runs the same seam through the C++ driver."""
    import shutil
    import subprocess
    ref_dir = os.environ.get("CPC_REFERENCE_DIR", "/root/reference")
    if not os.path.isdir(ref_dir) or shutil.which("g++") is None:
        pytest.skip("reference sources not present on this host")
    from corr_pc_gb300 import build as b
    if not os.path.exists(b.LIB):
        pytest.skip("library not built")
    odir = os.path.join(ROOT, "oracle", "_ref")
    os.makedirs(odir, exist_ok=True)
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "drop_in",
                        f"REF_DIR={ref_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    exe = os.path.join(odir, "corr_pc_gpu")
    syms = subprocess.run(["nm", "-C", exe], capture_output=True, text=True).stdout
    # the binding's corels2/corels1 are the ones do_corr calls; the reference's
    # CPU loops are still there under their new names
    for name in ("corels2(gal*, gal*, bin_jk&, data_info&)", "corels1(gal*, bin_jk&, data_info&)",
                 "corels2_cpu", "corels1_cpu"):
        assert name in syms, name
    needed = subprocess.run(["readelf", "-d", exe], capture_output=True, text=True).stdout
    assert "libcorrpc_gb300.so" in needed


def test_accuracy_report_applies_the_bar():
    """bench.py's per-field accuracy report: identical blocks pass; a changed
    count, a non-cancelling field off by 1e-5, or a cancelling field off by 1e-5
    relative in a bin holding more than 1% of its largest value fails; a
    cancelling bin near zero is held to the absolute floor."""
    from corr_pc_gb300 import metrics
    rng = np.random.default_rng(3)
    num = rng.integers(1, 1000, size=(3, 4, 5))
    sums = np.zeros((3, 4, 5, 13))
    sums[..., 0] = num
    sums[..., 1] = rng.normal(size=num.shape) * 10.0     # e+ sum: cancelling
    sums[..., 2] = rng.uniform(1.0, 2.0, num.shape) * num  # its square: non-cancelling
    rep = metrics.accuracy_report(num, sums, num, sums)
    assert rep["ok"] and rep["counts_bit_exact"]
    assert set(rep["fields"]) == {"wt_num", "data1.val", "data1.err"}
    bad_num = num.copy()
    bad_num[1, 2, 3] += 1
    assert not metrics.accuracy_report(bad_num, sums, num, sums)["ok"]
    worse = sums.copy()
    worse[..., 2] *= 1 + 1e-5
    assert not metrics.accuracy_report(num, worse, num, sums)["ok"]
    # a cancelling field: a bin near zero may be off relatively, within the floor
    canc = sums.copy()
    i = np.unravel_index(np.argmin(np.abs(sums[..., 1])), num.shape)
    canc[i + (1,)] += 1e-7 * np.abs(sums[..., 1]).max()
    rep = metrics.accuracy_report(num, canc, num, sums)
    assert rep["ok"] and rep["fields"]["data1.val"]["cancelling"]
    # ... but a bin holding 1% or more of its largest value is held to 1e-6 relative
    big = np.abs(sums[..., 1]) >= 0.01 * np.abs(sums[..., 1]).max()
    j = np.unravel_index(np.argmin(np.where(big, np.abs(sums[..., 1]), np.inf)), num.shape)
    canc = sums.copy()
    canc[j + (1,)] *= 1 + 1e-5
    assert not metrics.accuracy_report(num, canc, num, sums)["ok"]


@pytest.fixture(scope="module")
def asan_driver(tmp_path_factory):
    """tests/host_asan_driver.cpp and the C++ host sources, built with
    AddressSanitizer and UndefinedBehaviorSanitizer (once per module)."""
    import shutil
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    csrc = os.path.join(ROOT, "corr_pc_gb300", "csrc")
    exe = str(tmp_path_factory.mktemp("asan") / "host_asan_driver")
    srcs = [os.path.join(ROOT, "tests", "host_asan_driver.cpp")] + [
        os.path.join(csrc, s) for s in ("host/inp.cpp", "host/reader.cpp", "host/finalize.cpp",
                                        "host/outp.cpp", "host_helpers.cpp")]
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-pthread", "-fsanitize=address,undefined",
                        "-fno-sanitize-recover=all", "-fno-omit-frame-pointer",
                        "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
                        *srcs, "-o", exe], capture_output=True, text=True)
    if r.returncode != 0 and "asan" in (r.stderr or "").lower():
        pytest.skip("sanitizer runtime not available: " + r.stderr[-300:])
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("name", ["box_wgp_clustered", "box_wpp_weighted_distinct",
                                  "box_kappa_unsorted", "box_ed_rmu"])
def test_host_pipeline_under_address_and_ub_sanitizers(name, asan_driver, tmp_path):
    """The C++ host side of the command line (positional .inp, the catalogue
    readers with their rand() draws, the delete-one step, the finalisation and
    the output writers), built with AddressSanitizer and
    UndefinedBehaviorSanitizer and fed the reference's own raw SD block: it runs
    clean and writes the reference's output files."""
    g = Golden(name)
    wl = synth.Workload(name, g.params, g.S, g.D)
    inp = synth.write_box_run(str(tmp_path), wl, same_files=g.meta["same_files"], n_threads=1)
    nfile, sfile = str(tmp_path / "num.bin"), str(tmp_path / "sums.bin")
    np.ascontiguousarray(g.raw_num, dtype=np.int64).tofile(nfile)
    np.ascontiguousarray(g.raw_sums, dtype=np.float64).tofile(sfile)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:exitcode=23",
               UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([asan_driver, inp, nfile, sfile], capture_output=True, text=True,
                       env=env, timeout=300)
    if "LeakSanitizer has encountered a fatal error" in r.stderr:  # no ptrace here
        env["ASAN_OPTIONS"] = "detect_leaks=0:exitcode=23"
        r = subprocess.run([asan_driver, inp, nfile, sfile], capture_output=True, text=True,
                           env=env, timeout=300)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "runtime error" not in r.stderr, r.stderr[-4000:]
    # synth.write_box_run names the output prefix <dir>/out/run_
    for fname, ref in g.files.items():
        if fname.endswith(".info"):
            continue
        path = tmp_path / "out" / ("run_" + fname)
        assert path.exists(), fname
        compare_files(path.read_text(), ref, label=f"{name}:{fname} (sanitized host)")


def _run_sanitized(args):
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:exitcode=23",
               UBSAN_OPTIONS="print_stacktrace=1")
    return subprocess.run(args, capture_output=True, text=True, env=env, timeout=600)


def test_chunked_reader_under_sanitizers(asan_driver, tmp_path):
    """The C++ catalogue reader parses each file in ~1 MiB chunks on several
    threads and parses a file that S and D share once: on a 300k-galaxy box
    (files of 7-16 MB) it returns exactly the written values, the oracle's
    rand() draws and angles, and on a file with a bad value the row at which
    the sequential reader stops."""
    cat = synth.uniform_box(300000, 500.0, 11, nside_jk=4, with_shapes=True)
    p = synth._box_params(which_corr=1, L=500.0, rmin=0.1, rmax=60.0, nrp=20, npi=40,
                          pmax=100.0, njk=64, n=cat.n)
    inp = synth.write_box_run(str(tmp_path), synth.Workload("chunked", p, cat, cat))
    assert os.path.getsize(str(tmp_path / "S_pos.dat")) > 8 << 20
    out = str(tmp_path / "dump.bin")
    r = _run_sanitized([asan_driver, "--dump", inp, out])
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert "runtime error" not in r.stderr, r.stderr[-4000:]
    raw = open(out, "rb").read()
    ref = oracle.read_like_reference(p, [("S", cat), ("D", cat)])
    at = 0
    for role in ("S", "D"):
        n = int(np.frombuffer(raw, np.int64, 1, at)[0])
        at += 8
        assert n == cat.n
        cols = np.frombuffer(raw, np.float64, 8 * n, at).reshape(8, n)
        at += 64 * n
        jk = np.frombuffer(raw, np.int32, n, at)
        at += 4 * n
        e1, e2 = (np.zeros(n) if e is None else e for e in (ref[role].e1, ref[role].e2))
        assert (role == "S") == (ref[role].e1 is not None)  # D carries no shapes in wg+
        for k, want in enumerate((cat.x, cat.y, cat.z, np.ones(n), ref[role].phi,
                                  ref[role].jk_prob, e1, e2)):
            assert np.array_equal(cols[k], want), (role, k)
        assert np.array_equal(jk, cat.jk)
    # a value that is not a number in the middle of the z file: reading stops
    # at that row, as the sequential reader does
    zf = str(tmp_path / "S_z.dat")
    lines = open(zf).read().split("\n")
    bad_row = 171234
    lines[bad_row] = "x" + lines[bad_row]
    open(zf, "w").write("\n".join(lines))
    r = _run_sanitized([asan_driver, "--dump", inp, out])
    assert r.returncode == 1
    assert f"gal data reading ended unexpectedly at row {bad_row} " in r.stdout, r.stdout
    assert "runtime error" not in r.stderr
    # "inf" and "nan" tokens, which from_chars would accept and istream >> double
    # does not: reading stops at the first of them
    lines[bad_row] = lines[bad_row][1:]
    for tok, row in (("inf", 98765), ("-nan", 45678)):
        lines[row] = tok
        open(zf, "w").write("\n".join(lines))
        r = _run_sanitized([asan_driver, "--dump", inp, out])
        assert r.returncode == 1
        assert f"gal data reading ended unexpectedly at row {row} " in r.stdout, (tok, r.stdout)


def test_host_threads_under_thread_sanitizer(tmp_path):
    """The host side's threads (chunked parsing of the catalogue files, the
    output tables written in parallel) under ThreadSanitizer: no data race
    reported, and the reference's output files."""
    import shutil
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    csrc = os.path.join(ROOT, "corr_pc_gb300", "csrc")
    exe = str(tmp_path / "host_tsan_driver")
    srcs = [os.path.join(ROOT, "tests", "host_asan_driver.cpp")] + [
        os.path.join(csrc, s) for s in ("host/inp.cpp", "host/reader.cpp", "host/finalize.cpp",
                                        "host/outp.cpp", "host_helpers.cpp")]
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-pthread", "-fsanitize=thread",
                        "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
                        *srcs, "-o", exe], capture_output=True, text=True)
    if r.returncode != 0 and "tsan" in (r.stderr or "").lower():
        pytest.skip("thread sanitizer runtime not available: " + r.stderr[-300:])
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, TSAN_OPTIONS="halt_on_error=1:exitcode=66")
    # a 300k-galaxy box: files of several MiB, parsed in chunks
    cat = synth.uniform_box(300000, 500.0, 5, nside_jk=3, with_shapes=True)
    p = synth._box_params(which_corr=2, L=500.0, rmin=0.1, rmax=60.0, nrp=20, npi=40,
                          pmax=100.0, njk=27, n=cat.n)
    big = tmp_path / "big"
    inp = synth.write_box_run(str(big), synth.Workload("tsan", p, cat, cat))
    r = subprocess.run([exe, "--dump", inp, str(big / "dump.bin")], capture_output=True,
                       text=True, env=env, timeout=600)
    if "FATAL: ThreadSanitizer" in r.stderr:
        pytest.skip("thread sanitizer cannot run here: " + r.stderr[-300:])
    assert r.returncode == 0 and "WARNING: ThreadSanitizer" not in r.stderr, r.stderr[-4000:]
    # a golden run with jackknife regions: every output table written in parallel
    g = Golden("box_wgp_clustered")
    run = tmp_path / "golden"
    inp = synth.write_box_run(str(run), synth.Workload("g", g.params, g.S, g.D),
                              same_files=g.meta["same_files"], n_threads=1)
    nfile, sfile = str(run / "num.bin"), str(run / "sums.bin")
    np.ascontiguousarray(g.raw_num, dtype=np.int64).tofile(nfile)
    np.ascontiguousarray(g.raw_sums, dtype=np.float64).tofile(sfile)
    r = subprocess.run([exe, inp, nfile, sfile], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0 and "WARNING: ThreadSanitizer" not in r.stderr, r.stderr[-4000:]
    n_files = 0
    for fname, ref in g.files.items():
        if fname.endswith(".info"):
            continue
        compare_files((run / "out" / ("run_" + fname)).read_text(), ref,
                      label=f"{fname} (thread sanitizer)")
        n_files += 1
    assert n_files > 0
    # 27 regions x 10 tables, the full-sample and jackknife-final tables, temporaries
    assert len(os.listdir(run / "out")) > 27 * 10


def test_unwritable_output_prefix_is_an_error(asan_driver, tmp_path):
    """Output tables written in parallel: one that cannot be opened still makes
    the finalisation fail with the writer's message."""
    g = Golden("box_wgp_clustered")
    wl = synth.Workload("g", g.params, g.S, g.D)
    inp = synth.write_box_run(str(tmp_path), wl, same_files=g.meta["same_files"], n_threads=1)
    p = synth.InpParams.read(inp)
    p.out_file = str(tmp_path / "missing_dir" / "run_")
    p.write(inp)
    nfile, sfile = str(tmp_path / "num.bin"), str(tmp_path / "sums.bin")
    np.ascontiguousarray(g.raw_num, dtype=np.int64).tofile(nfile)
    np.ascontiguousarray(g.raw_sums, dtype=np.float64).tofile(sfile)
    r = _run_sanitized([asan_driver, inp, nfile, sfile])
    assert r.returncode == 1, (r.stdout, r.stderr[-2000:])
    assert "could not write output files with prefix" in r.stdout
    assert "runtime error" not in r.stderr
