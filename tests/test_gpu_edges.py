"""Entry points at their edges, through the C ABI: node and edge counts at
the int32 limit refused from the scalars alone, and a solve's scores left on
the device and read there by top_k."""
import ctypes

import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300 import _native, gen
from graphops_gb300.topk import top_k_device

pytestmark = pytest.mark.gpu


def upload(rp, col):
    return go.DeviceGraph.from_csr(np.array(rp, np.int64), np.array(col, np.int32))


def ref_top_k(x, k):
    ok = np.isfinite(x) & (x > 0)
    cand = np.nonzero(ok)[0]
    return sorted(cand.tolist(), key=lambda i: (-x[i], i))[:k]


def test_size_limits_refused_from_the_scalars():
    """n and m must stay below 2^31 - 1 (int32 indices in the device CSR).
    Both are refused from the scalars alone: n before row_ptr is read, m
    (= row_ptr[n]) before col is read, so the tiny arrays here are never read
    past their ends and nothing reaches the device."""
    ctx = _native.default_context()
    lib = ctx._l
    col = np.zeros(1, np.int32)
    for n, rp, msg in ((2**31 - 1, np.zeros(1, np.int64), "node count out of range"),
                       (2**40, np.zeros(1, np.int64), "node count out of range"),
                       (1, np.array([0, 2**31 - 1], np.int64), "edge count out of range")):
        h = ctypes.c_void_p()
        rc = lib.gops_graph_upload(ctx.handle, n, _native.ptr(rp), _native.ptr(col), None, ctypes.byref(h))
        assert rc == _native.GOPS_ERR_INVALID and h.value is None
        assert lib.gops_last_error(ctx.handle).decode() == msg
    g = upload([0, 1, 2, 2], [1, 2])  # the context is still usable
    assert g.pagerank_run(go.PageRankConfig())[3]


def test_solve_left_on_device_then_top_k_there():
    """A solve without a host buffer leaves its scores on the device
    (gops_ctx_scores_device), where top_k reads them: the same entries as the
    host copy of the same (bitwise-repeatable) solve.  The context's counters
    show the one copy to the host."""
    g = gen.rmat(12, 16, weighted=True, seed=12)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col, g.weight.astype(np.float64))
    conf = go.PageRankConfig(0.85, 1000, 1e-8)
    s, it, _, conv = dg.pagerank_weighted_run(conf)
    st = dg.ctx.stats()
    assert conv and st.d2h_bytes == 8 * g.n and st.kernel_launches > 0
    _, it2, _, _ = dg.pagerank_weighted_run(conf, out=False)
    assert it2 == it and dg.ctx.stats().d2h_bytes == 0
    ptr = dg.ctx._l.gops_ctx_scores_device(dg.ctx.handle)
    assert ptr
    got = top_k_device(ptr, g.n, 100, ctx=dg.ctx)
    want = ref_top_k(s, 100)
    assert [i for i, _ in got] == want and [v for _, v in got] == [s[i] for i in want]
