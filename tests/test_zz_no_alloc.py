"""cpc_count_fp64_noalloc: the counting entry point for callers that cannot
allocate GPU memory (embedded in applications whose framework or memory pool
owns every device allocation).  Its scratch is a fixed array inside the
library; the inputs and outputs here are device buffers this test allocates
on the caller's side (with torch).  The result must equal the regular entry
point's, on two calls in a row (the second call reuses the scratch the first
one left behind)."""
import numpy as np
import pytest

from corr_pc_gb300 import _lib, host
from helpers import Golden, check_sums

pytestmark = pytest.mark.gpu


def _device_catalog(torch, g):
    keep = []

    def put(a, dt):
        if a is None:
            return None
        t = torch.tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
        keep.append(t)
        return t.data_ptr()

    d = {"n": g.n, "x": put(g.x, torch.float64), "y": put(g.y, torch.float64),
         "z": put(g.z, torch.float64), "w": put(g.w, torch.float64),
         "e1": put(g.e1, torch.float64), "e2": put(g.e2, torch.float64),
         "phi": put(g.phi, torch.float64), "jk_prob": put(g.jk_prob, torch.float64),
         "jk": put(g.jk, torch.int32)}
    return d, keep


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
    nh, nb, npb = ctx.shape
    d_num = torch.empty(nh * nb * npb, dtype=torch.int64, device="cuda")
    d_sums = torch.empty(nh * nb * npb * _lib.NF, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        d_num.fill_(-7)   # the call must zero its outputs itself
        d_sums.fill_(3.0)
        r = _lib.count_fp64_noalloc(p, "SD", d1, d2, d_num.data_ptr(), d_sums.data_ptr(), stream)
        torch.cuda.synchronize()
        num = d_num.cpu().numpy().reshape(nh, nb, npb)
        sums = d_sums.cpu().numpy().reshape(nh, nb, npb, _lib.NF)
        assert r["n_binned"] == ref["n_binned"] == g.n_in
        assert r["n_window"] == ref["n_window"] == g.n_total
        assert np.array_equal(num, ref["num"])
        check_sums(sums, ref["sums"], label="noalloc")
    del k1, k2
