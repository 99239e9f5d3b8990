"""cpc_count_fp64_noalloc: the counting entry point for callers that cannot
allocate GPU memory (embedded in applications whose framework or memory pool
owns every device allocation).  Its scratch is a fixed array inside the
library; the inputs and outputs here are device buffers this test allocates
on the caller's side (with torch).  The result must equal the regular entry
point's and the reference's own histograms (the golden fixture), on two calls
in a row (the second call reuses the scratch the first one left behind); bad
inputs are rejected before any pair is counted, and a clean call after them
still matches."""
import numpy as np
import pytest

from corr_pc_gb300 import _lib, host
from helpers import Golden, check_sums

pytestmark = pytest.mark.gpu


def _device_catalog(torch, g, **override):
    keep = []

    def put(a, dt):
        if a is None:
            return None
        t = torch.tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
        keep.append(t)
        return t.data_ptr()

    src = {"x": g.x, "y": g.y, "z": g.z, "w": g.w, "e1": g.e1, "e2": g.e2, "phi": g.phi,
           "jk_prob": g.jk_prob, "jk": g.jk}
    src.update(override)
    d = {"n": g.n}
    for k, v in src.items():
        d[k] = put(v, torch.int32 if k == "jk" else torch.float64)
    return d, keep


def _outputs(torch, ctx):
    nh, nb, npb = ctx.shape
    d_num = torch.empty(nh * nb * npb, dtype=torch.int64, device="cuda")
    d_sums = torch.empty(nh * nb * npb * _lib.NF, dtype=torch.float64, device="cuda")
    return d_num, d_sums


def _run(torch, ctx, p, d1, d2, d_num, d_sums):
    nh, nb, npb = ctx.shape
    d_num.fill_(-7)   # the call must zero its outputs itself
    d_sums.fill_(3.0)
    stream = torch.cuda.current_stream().cuda_stream
    r = _lib.count_fp64_noalloc(p, "SD", d1, d2, d_num.data_ptr(), d_sums.data_ptr(), stream)
    torch.cuda.synchronize()
    num = d_num.cpu().numpy().reshape(nh, nb, npb)
    sums = d_sums.cpu().numpy().reshape(nh, nb, npb, _lib.NF)
    return r, num, sums


@pytest.mark.parametrize("name", ["box_wpp_weighted_distinct", "box_wgp_clustered"])
def test_noalloc_matches_regular_entry_point_twice(name):
    torch = pytest.importorskip("torch")
    g = Golden(name)
    p = g.params
    cats = host.prepare(p, [("S", g.S), ("D", g.D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    ref = ctx.count("SD", 0, 1, engine="fp64")
    d1, k1 = _device_catalog(torch, cats["D"])
    d2, k2 = _device_catalog(torch, cats["S"])
    d_num, d_sums = _outputs(torch, ctx)
    for _ in range(2):
        r, num, sums = _run(torch, ctx, p, d1, d2, d_num, d_sums)
        assert r["n_binned"] == ref["n_binned"] == g.n_in
        assert r["n_window"] == ref["n_window"] == g.n_total
        assert np.array_equal(num, ref["num"])
        assert np.array_equal(num, g.raw_num)
        check_sums(sums, ref["sums"], label="noalloc vs regular")
        check_sums(sums, g.raw_sums, label="noalloc vs reference")
    del k1, k2


def test_noalloc_swap_rule_matches_regular_entry_point():
    """The catalogues in the other order: the smaller one first, so the swap
    rule (corr.cpp:281-296) exchanges them and the shape holder."""
    torch = pytest.importorskip("torch")
    g = Golden("box_wgp_swap")
    p = g.params
    cats = host.prepare(p, [("S", g.S), ("D", g.D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    for a, b in ((0, 1), (1, 0)):
        ref = ctx.count("SD", a, b, engine="fp64")
        ga, gb = (cats["D"], cats["S"]) if a == 0 else (cats["S"], cats["D"])
        d1, k1 = _device_catalog(torch, ga)
        d2, k2 = _device_catalog(torch, gb)
        d_num, d_sums = _outputs(torch, ctx)
        r, num, sums = _run(torch, ctx, p, d1, d2, d_num, d_sums)
        assert r["n_binned"] == ref["n_binned"]
        assert np.array_equal(num, ref["num"])
        check_sums(sums, ref["sums"], label=f"swap order {a}{b}")
        del k1, k2


def test_noalloc_rejects_bad_inputs_then_counts_cleanly():
    """An unsorted scanned catalogue, a jackknife label out of range and a
    missing jk_prob are rejected with status codes (detected before the count
    kernel runs); the next clean call still equals the regular entry point,
    whatever the rejected calls left in the shared scratch."""
    torch = pytest.importorskip("torch")
    g = Golden("box_wgp_clustered")
    p = g.params
    cats = host.prepare(p, [("S", g.S), ("D", g.D)])
    ctx = _lib.Context(p)
    ctx.upload(0, cats["D"])
    ctx.upload(1, cats["S"])
    ref = ctx.count("SD", 0, 1, engine="fp64")
    d1, k1 = _device_catalog(torch, cats["D"])
    d_num, d_sums = _outputs(torch, ctx)
    s = cats["S"]
    z_rev = np.ascontiguousarray(s.z[::-1])
    bad_z, kz = _device_catalog(torch, s, z=z_rev)
    jk_bad = np.array(s.jk, dtype=np.int32)
    jk_bad[len(jk_bad) // 2] = p.n_jk_regions  # one past the last region
    bad_jk, kj = _device_catalog(torch, s, jk=jk_bad)
    no_prob, kp = _device_catalog(torch, s, jk_prob=None)
    for cat, status in ((bad_z, "CPC_ERR_INVALID"), (bad_jk, "CPC_ERR_RANGE"),
                        (no_prob, "CPC_ERR_INVALID")):
        with pytest.raises(_lib.CpcError) as ei:
            _run(torch, ctx, p, d1, cat, d_num, d_sums)
        assert _lib.STATUS_NAMES[ei.value.status] == status, str(ei.value)
    d2, k2 = _device_catalog(torch, s)
    r, num, sums = _run(torch, ctx, p, d1, d2, d_num, d_sums)
    assert r["n_binned"] == ref["n_binned"]
    assert np.array_equal(num, ref["num"])
    check_sums(sums, ref["sums"], label="clean call after rejected ones")
    del k1, k2, kz, kj, kp
