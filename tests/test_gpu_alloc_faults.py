"""Allocation failures, injected on the host (gops_debug_fail_allocations_after):
every device allocation of the library's pool in turn fails as if the device
were out of memory.  Each call must either succeed or report GOPS_ERR_OOM,
leave the context usable, and leave no half-built graph, workspace or batch
state behind: with injection off again, the same objects solve correctly.
No GPU fault is involved (the allocation is refused before CUDA is asked)."""
import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300 import _native, gen
from graphops_gb300._native import GopsError, GOPS_ERR_OOM
from oracle import port

pytestmark = pytest.mark.gpu


def hook(count):
    _native.lib().gops_debug_fail_allocations_after(int(count))


@pytest.fixture(autouse=True)
def _hook_off():
    yield
    hook(-1)


def test_every_allocation_failure_is_reported_and_recoverable():
    g = gen.rmat(12, 16, weighted=True, seed=12)
    w = g.weight.astype(np.float64)
    conf = go.PageRankConfig(0.85, 1000, 1e-8)
    ref = port.pagerank_weighted_run(g.row_ptr, g.col, w, 0.85, 1000, 1e-8)
    sp, si = gen.seed_sets(g, 40, 1, 16, seed=3)
    ok_runs = oom_upload = oom_later = 0
    for k in range(0, 200):
        hook(k)
        dg = None
        try:
            dg = go.DeviceGraph.from_csr(g.row_ptr, g.col, w)
            dg.pagerank_weighted_run(conf)
            dg.ppr_batch(conf, sp, si, out=True)
            ok_runs += 1
            break  # k allocations were enough for everything
        except GopsError as e:
            assert e.code == GOPS_ERR_OOM, e
            if dg is None:
                oom_upload += 1
            else:
                oom_later += 1
        hook(-1)
        # whatever was built before the failure is sound: solve it now
        if dg is not None:
            s, it, _, conv = dg.pagerank_weighted_run(conf)
            assert conv and it == ref[1] and np.abs(s - ref[0]).sum() <= 1e-7
            scores = dg.ppr_batch(conf, sp, si, out=True)[0]
            assert np.isfinite(scores).all() and np.abs(scores.sum(axis=1) - 1.0).max() < 1e-5
    hook(-1)
    assert ok_runs == 1  # some count lets every allocation through
    # failures were injected into the upload and into the solve / batch
    assert oom_upload >= 10 and oom_later >= 3, (oom_upload, oom_later)
    # and a fresh upload after all of it
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col, w)
    s, it, _, conv = dg.pagerank_weighted_run(conf)
    assert conv and it == ref[1] and np.abs(s - ref[0]).sum() <= 1e-7
