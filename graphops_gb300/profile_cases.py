"""One small case per kernel family, for profiling a single kernel in isolation
(e.g. under ncu with a kernel filter): each case builds its graph, runs a
few warm-up calls and then the profiled call.  Inputs are larger than the
GPU's L2 cache (so DRAM figures mean something) while the whole case holds a
few GB of device memory at most.

    python -m graphops_gb300.profile_cases <case>

cases:
  pagerank   weighted PageRank, R-MAT scale 21 (2 M nodes, ~32 M edges), tol 1e-8:
             iterate_kernel (double-float and FP32 steps), init / finalize
  upload     the out-CSR upload and device build of that graph (radix sort,
             scatter_edges, the per-row weight passes)
  upload22   the same for an R-MAT scale 22 graph (4 M nodes, ~65 M edges),
             uploaded from pinned host arrays three times
  batched    batched PPR on R-MAT scale 20, one wave of 128 seed sets (the
             bench's k-tile): spmm_mixed and spmm_f32
  centrality Katz, eigenvector centrality and HITS on R-MAT scale 21
  topk       top-100 of a 2 M-entry FP64 score vector and of 128 FP32 rows
  warm       the warm start's network on a stochastic block model (n = 500,000):
             three loss / gradient evaluations of 16 sets, each one forward
             (layer 1, aggregation, the tcgen05 layer 2) and one backward
             (the tcgen05 input gradient, the weight-gradient reductions)
"""
from __future__ import annotations

import sys

import numpy as np


def _rmat(scale, weighted=False, seed=21):
    from . import gen
    return gen.rmat(scale, 16, 0.57, 0.19, 0.19, weighted=weighted, wlo=0.1, whi=1.0, seed=seed)


def case_pagerank():
    from . import _native
    from .pagerank import PageRankConfig
    g = _rmat(21, weighted=True)
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col, g.weight.astype(np.float64))
    conf = PageRankConfig(0.85, 1000, 1e-8)
    for _ in range(3):
        dg.pagerank_weighted_run(conf, out=False)
    dg.pagerank_weighted_run(conf, out=True)


def case_upload():
    from . import _native
    g = _rmat(21, weighted=True)
    w = g.weight.astype(np.float64)
    for _ in range(3):
        _native.DeviceGraph.from_csr(g.row_ptr, g.col, w).close()


def case_upload22():
    """An R-MAT 22 graph with FP64 weights (the bench's weighted PageRank
    sizes) uploaded from pinned host arrays three times."""
    import torch
    from . import _native
    g = _rmat(22, weighted=True, seed=22)
    rp = torch.from_numpy(g.row_ptr).pin_memory().numpy()
    col = torch.from_numpy(g.col).pin_memory().numpy()
    w = torch.from_numpy(g.weight.astype(np.float64)).pin_memory().numpy()
    for _ in range(3):
        _native.DeviceGraph.from_csr(rp, col, w).close()
        torch.cuda.synchronize()


def case_batched():
    from . import _native, gen
    from .pagerank import PageRankConfig
    g = _rmat(20, seed=20)
    sp, si = gen.seed_sets(g, 128, 1, 64, seed=7)
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col)
    dg.set_batch_tile(128, 256, False)
    conf = PageRankConfig(0.85, 1000, 1e-7)
    for _ in range(2):
        dg.ppr_batch(conf, sp, si, out=False)


def case_centrality():
    from . import _native
    g = _rmat(21)
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col)
    for _ in range(2):
        dg.katz_run(1e-4, 1.0, 100, 1e-10, out=False)
        dg.eigenvector_run(100, 1e-8, out=False)
        dg.hits_run(100, 1e-8)


def case_topk():
    import torch
    from . import _native
    from .topk import top_k_device, top_k_rows_device
    ctx = _native.default_context()
    n = 1 << 21
    rng = np.random.default_rng(3)
    x = torch.from_numpy(rng.random(n)).to("cuda")
    rows = torch.from_numpy(rng.random((128, n), dtype=np.float32)).to("cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        top_k_device(x.data_ptr(), n, 100, ctx=ctx)
        top_k_rows_device(rows.data_ptr(), 128, n, 100, ctx=ctx)


def case_warm():
    from . import _native, gen, warm
    g = gen.sbm(500000, 64, 1.2, 16.0, 4.0, seed=3)
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col)
    model = warm.WarmStart(dg, g.row_ptr, g.col, warm.default_config(clusters=72))
    sp, si = gen.seed_sets(g, 16, 1, 32, seed=11)
    rng = np.random.default_rng(5)
    t = rng.random((16, g.n), dtype=np.float32)
    t /= t.sum(axis=1, keepdims=True)
    for _ in range(3):
        model.loss_grad(0.85, sp, si, t)


CASES = {"pagerank": case_pagerank, "upload": case_upload, "upload22": case_upload22, "batched": case_batched,
         "centrality": case_centrality, "topk": case_topk, "warm": case_warm}


def main(argv):
    if len(argv) != 2 or argv[1] not in CASES:
        print(__doc__)
        return 2
    CASES[argv[1]]()
    print(f"case {argv[1]} done")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
