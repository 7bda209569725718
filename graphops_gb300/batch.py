"""Batched personalized PageRank: many seed sets in one pass over the graph.

Each seed set is exactly one ``personalized_pagerank_run`` of the reference
(src/ppr.rs:90-156) with personalization 1 on every seed node (a repeated
node counts twice), normalised by its sum -- an empty set means the uniform
vector (src/ppr.rs:104-109).  Each set stops at its own first step whose L1
norm falls below ``config.tolerance``.  Results are FP32 vectors.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _native
from .pagerank import PageRankConfig


@dataclass
class BatchRun:
    scores: Optional[np.ndarray]  # float32 [nsets, n], or None
    iterations: np.ndarray        # per set
    diff_l1: np.ndarray
    converged: np.ndarray


def seed_sets_to_csr(seed_sets: Sequence[Sequence[int]]):
    """[[nodes of set 0], [nodes of set 1], ...] -> (seed_ptr, seed_idx)."""
    ptr = np.zeros(len(seed_sets) + 1, dtype=np.int64)
    for i, s in enumerate(seed_sets):
        ptr[i + 1] = ptr[i] + len(s)
    idx = np.fromiter((int(v) for s in seed_sets for v in s), dtype=np.int32, count=int(ptr[-1]))
    return ptr, idx


def ppr_batch(graph, config: PageRankConfig, seed_ptr, seed_idx, x0=None,
              scores: bool = True) -> BatchRun:
    """Batched PPR on a DeviceGraph (or any adapter, uploaded first).

    ``x0`` (optional, float32 [nsets, n]) is a warm start replacing p as the
    start vector; the iteration and its stopping rule are unchanged."""
    from .pagerank import _device_graph
    config = config or PageRankConfig()
    dg = graph if isinstance(graph, _native.DeviceGraph) else _device_graph(graph, weighted=False)
    s, its, diffs, conv = dg.ppr_batch(config, seed_ptr, seed_idx, x0=x0, out=scores)
    return BatchRun(s, its, diffs, conv)
