"""gops_pagerank_run_noalloc against gops_pagerank_run, through the C ABI.

The no-allocation entry point serves callers that cannot allocate device
memory when they solve (their device memory belongs to another allocator, or
cudaMalloc would stall a latency-critical path).  It runs the same kernels on
a fixed scratch array inside the library, so its output must equal the
regular entry point's.  Two calls in a row check that the shared scratch,
which keeps the previous call's contents, is reset correctly.

This file sorts after the parity, batch, warm-start and upload tests, so that
a run stopping at the first failure has already run them; it passes alone in
a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

from graphops_gb300 import _native, gen

pytestmark = pytest.mark.gpu

L1_TOL = 1e-8  # the fixture bar of the parity tests; the two paths are expected to agree bit for bit


def _run(ctx, lib, fn, g, cfg):
    out = np.empty(g.n, dtype=np.float64)
    r = _native.Run()
    rc = getattr(lib, fn)(ctx.handle, g.handle, ctypes.byref(cfg), _native.ptr(out), ctypes.byref(r))
    return rc, out, r


def test_noalloc_matches_regular_entry_point_twice():
    ctx = _native.Context(0)
    lib = ctx._l
    cfg = _native.Config(0.85, 1000, 1e-9)
    graphs = [gen.rmat(16, 16, seed=3), gen.erdos_renyi(2000, 0.005, 0.01, seed=0)]
    for gg in graphs:
        g = _native.DeviceGraph.from_csr(gg.row_ptr, gg.col, ctx=ctx)
        rc, ref, rr = _run(ctx, lib, "gops_pagerank_run", g, cfg)
        assert rc == 0, lib.gops_last_error(ctx.handle)
        for _ in range(2):
            rc, out, r = _run(ctx, lib, "gops_pagerank_run_noalloc", g, cfg)
            assert rc == 0, lib.gops_last_error(ctx.handle)
            assert np.abs(out - ref).sum() <= L1_TOL
            assert (r.iterations, r.converged) == (rr.iterations, rr.converged)
            assert abs(r.diff_l1 - rr.diff_l1) <= 1e-12 * max(rr.diff_l1, 1e-300)
        g.close()
    ctx.close()


def test_noalloc_rejects_graphs_beyond_its_limit():
    ctx = _native.Context(0)
    lib = ctx._l
    n = (1 << 18) + 1
    g = _native.DeviceGraph.from_csr(np.zeros(n + 1, np.int64), np.zeros(0, np.int32), ctx=ctx)
    rc, out, r = _run(ctx, lib, "gops_pagerank_run_noalloc", g, _native.Config(0.85, 10, 1e-6))
    assert rc == _native.GOPS_ERR_INVALID
    assert b"too large" in lib.gops_last_error(ctx.handle)
    g.close()
    ctx.close()
