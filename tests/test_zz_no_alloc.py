"""gops_pagerank_run_noalloc against gops_pagerank_run, through the C ABI.

The no-allocation entry point serves callers that cannot allocate device
memory when they solve (their device memory belongs to another allocator, or
cudaMalloc would stall a latency-critical path).  It runs the same kernels on
a fixed scratch array inside the library, so its output must equal the
regular entry point's.  Two calls in a row check that the shared scratch,
which keeps the previous call's contents, is reset correctly.  With the
library's allocation hook armed to refuse every device allocation, the
regular entry point on a fresh graph fails (its workspace cannot be made)
while the no-alloc one still solves: it asks for no device memory.

This file sorts after every other test file, so that a run stopping at the
first failure has already run them; it passes alone in a fresh process as
well.
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


def test_noalloc_solves_with_every_allocation_refused():
    ctx = _native.Context(0)
    lib = ctx._l
    cfg = _native.Config(0.85, 1000, 1e-9)
    gg = gen.rmat(15, 16, seed=4)
    g1 = _native.DeviceGraph.from_csr(gg.row_ptr, gg.col, ctx=ctx)
    rc, ref, rr = _run(ctx, lib, "gops_pagerank_run", g1, cfg)
    assert rc == 0, lib.gops_last_error(ctx.handle)
    g2 = _native.DeviceGraph.from_csr(gg.row_ptr, gg.col, ctx=ctx)  # no workspace yet
    lib.gops_debug_fail_allocations_after(0)
    try:
        rc_regular, _, _ = _run(ctx, lib, "gops_pagerank_run", g2, cfg)
        runs = [_run(ctx, lib, "gops_pagerank_run_noalloc", g2, cfg) for _ in range(2)]
    finally:
        lib.gops_debug_fail_allocations_after(-1)
    assert rc_regular == _native.GOPS_ERR_OOM
    for rc, out, r in runs:
        assert rc == 0, lib.gops_last_error(ctx.handle)
        assert np.abs(out - ref).sum() <= L1_TOL
        assert (r.iterations, r.converged) == (rr.iterations, rr.converged)
    g1.close()
    g2.close()
    ctx.close()


def test_noalloc_rejects_graphs_beyond_its_node_limit():
    ctx = _native.Context(0)
    lib = ctx._l
    n = (1 << 18) + 1
    g = _native.DeviceGraph.from_csr(np.zeros(n + 1, np.int64), np.zeros(0, np.int32), ctx=ctx)
    rc, out, r = _run(ctx, lib, "gops_pagerank_run_noalloc", g, _native.Config(0.85, 10, 1e-6))
    assert rc == _native.GOPS_ERR_INVALID
    assert b"too large" in lib.gops_last_error(ctx.handle)
    g.close()
    ctx.close()


def test_noalloc_rejects_graphs_beyond_its_hub_task_limit():
    """Fewer nodes than the limit, but 17 rows of 4,000,000 in-edges each
    (every node points 20 times at each of nodes 0..16): 17 x 3,907 hub tasks
    of 1,024 edges = 66,419 > 65,536, whose partials would not fit in the
    scratch array's hub slots."""
    ctx = _native.Context(0)
    lib = ctx._l
    n, hubs, rep = 200000, 17, 20
    row = np.repeat(np.arange(hubs, dtype=np.int32), rep)
    col = np.tile(row, n)
    rp = np.arange(n + 1, dtype=np.int64) * row.shape[0]
    g = _native.DeviceGraph.from_csr(rp, col, ctx=ctx)
    rc, out, r = _run(ctx, lib, "gops_pagerank_run_noalloc", g, _native.Config(0.85, 10, 1e-6))
    assert rc == _native.GOPS_ERR_INVALID
    err = lib.gops_last_error(ctx.handle)
    assert b"too large" in err and b"hub tasks=66419" in err, err
    g.close()
    ctx.close()
