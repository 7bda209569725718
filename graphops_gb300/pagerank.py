"""PageRank and personalized PageRank, mirroring graphops' public API.

Reference: src/pagerank.rs (PageRankRun :14-29, PageRankConfig :37-86,
pagerank* :91-336) and src/ppr.rs (personalized_pagerank* :11-156).  Same
names, same argument meaning, same validation messages, same results (within
the tolerances the tests state) -- computed by libgops on the GPU.

Graph arguments are adapters (see :mod:`graphops_gb300.graph`) or a
:class:`~graphops_gb300._native.DeviceGraph` already resident on the device
(which skips the upload, for repeated solves on one graph).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import List, Sequence

import numpy as np

from . import _native
from .graph import AdjacencyMatrix, DiGraph, extract


class GraphopsError(Exception):
    """Errors of the *_checked variants (src/lib.rs:108-123)."""


class InvalidParameter(GraphopsError):
    def __init__(self, msg: str):
        super().__init__(f"invalid parameter: {msg}")
        self.msg = msg


@dataclass
class PageRankConfig:
    """Hyperparameters (src/pagerank.rs:39-59); defaults 0.85 / 100 / 1e-6."""
    damping: float = 0.85
    max_iterations: int = 100
    tolerance: float = 1e-6

    def validate(self) -> None:
        """src/pagerank.rs:63-85, with the reference's messages."""
        if not math.isfinite(self.damping):
            raise InvalidParameter("damping must be finite")
        if not (0.0 <= self.damping <= 1.0):
            raise InvalidParameter("damping must be in [0,1]")
        if self.max_iterations == 0:
            raise InvalidParameter("max_iterations must be > 0")
        if not math.isfinite(self.tolerance) or self.tolerance <= 0.0:
            raise InvalidParameter("tolerance must be finite and > 0")


@dataclass
class PageRankRun:
    """Scores plus convergence diagnostics (src/pagerank.rs:16-29)."""
    scores: np.ndarray
    iterations: int
    diff_l1: float
    converged: bool


def _device_graph(graph, weighted: bool) -> "_native.DeviceGraph":
    if isinstance(graph, _native.DeviceGraph):
        return graph
    if isinstance(graph, AdjacencyMatrix):
        return _native.DeviceGraph.from_dense(graph.matrix)
    if isinstance(graph, DiGraph):  # bulk: the raw edge list, built on the device
        src, dst, w = graph.raw_edges()
        return _native.DeviceGraph.from_edges(graph.node_count(), src, dst, w if weighted else None)
    rp, col, w = extract(graph, weighted)
    return _native.DeviceGraph.from_csr(rp, col, w)


def _empty_run() -> PageRankRun:
    return PageRankRun(np.zeros(0), 0, 0.0, True)


def _n(graph) -> int:
    return graph.n if isinstance(graph, _native.DeviceGraph) else graph.node_count()


# ---- unweighted ----------------------------------------------------------

def pagerank_run(graph, config: PageRankConfig = None) -> PageRankRun:
    """src/pagerank.rs:122-187."""
    config = config or PageRankConfig()
    if _n(graph) == 0:
        return _empty_run()
    dg = _device_graph(graph, weighted=False)
    s, it, diff, conv = dg.pagerank_run(config)
    return PageRankRun(s, it, diff, conv)


def pagerank(graph, config: PageRankConfig = None) -> np.ndarray:
    """src/pagerank.rs:114-116."""
    return pagerank_run(graph, config).scores


def pagerank_checked(graph, config: PageRankConfig = None) -> np.ndarray:
    """src/pagerank.rs:91-94."""
    config = config or PageRankConfig()
    config.validate()
    return pagerank(graph, config)


def pagerank_checked_run(graph, config: PageRankConfig = None) -> PageRankRun:
    """src/pagerank.rs:321-324."""
    config = config or PageRankConfig()
    config.validate()
    return pagerank_run(graph, config)


# ---- weighted ------------------------------------------------------------

def pagerank_weighted_run(graph, config: PageRankConfig = None) -> PageRankRun:
    """src/pagerank.rs:210-289 (negative weights clamp to 0)."""
    config = config or PageRankConfig()
    if _n(graph) == 0:
        return _empty_run()
    dg = _device_graph(graph, weighted=True)
    s, it, diff, conv = dg.pagerank_weighted_run(config)
    return PageRankRun(s, it, diff, conv)


def pagerank_weighted(graph, config: PageRankConfig = None) -> np.ndarray:
    """src/pagerank.rs:201-203."""
    return pagerank_weighted_run(graph, config).scores


def _check_weights(graph) -> None:
    """The weight loop of src/pagerank.rs:299-314."""
    if isinstance(graph, _native.DeviceGraph):
        return
    n = graph.node_count()
    for u in range(n):
        for v in graph.neighbors(u):
            w = graph.edge_weight(u, v)
            if not math.isfinite(w):
                raise InvalidParameter("edge weights must be finite")
            if w < 0.0:
                raise InvalidParameter("edge weights must be non-negative")


def pagerank_weighted_checked(graph, config: PageRankConfig = None) -> np.ndarray:
    """src/pagerank.rs:294-316."""
    config = config or PageRankConfig()
    config.validate()
    _check_weights(graph)
    return pagerank_weighted(graph, config)


def pagerank_weighted_checked_run(graph, config: PageRankConfig = None) -> PageRankRun:
    """src/pagerank.rs:328-336 (validates, then one solve: the reference's
    discarded first solve returns the same scores, so it is not repeated)."""
    config = config or PageRankConfig()
    config.validate()
    _check_weights(graph)
    return pagerank_weighted_run(graph, config)


# ---- personalized --------------------------------------------------------

def personalized_pagerank_run(graph, config: PageRankConfig, personalization: Sequence[float]) -> PageRankRun:
    """src/ppr.rs:90-156.  Unchecked: like the reference, it assumes
    len(personalization) == node_count (a mismatch raises IndexError here
    where the reference would panic on the slice index)."""
    config = config or PageRankConfig()
    n = _n(graph)
    if n == 0:
        return _empty_run()
    p = np.ascontiguousarray(personalization, dtype=np.float64)
    if p.shape[0] < n:
        raise IndexError("personalization shorter than node_count")
    dg = _device_graph(graph, weighted=False)
    s, it, diff, conv = dg.personalized_pagerank_run(config, p[:n])
    return PageRankRun(s, it, diff, conv)


def personalized_pagerank(graph, config: PageRankConfig, personalization: Sequence[float]) -> np.ndarray:
    """src/ppr.rs:66-72."""
    return personalized_pagerank_run(graph, config, personalization).scores


def _check_personalization(graph, config: PageRankConfig, personalization) -> None:
    """src/ppr.rs:16-42, with the reference's messages."""
    config.validate()
    n = _n(graph)
    p = list(personalization)
    if len(p) != n:
        raise InvalidParameter(
            f"personalization length must equal node_count (len={len(p)} node_count={n})")
    for x in p:
        if not math.isfinite(x):
            raise InvalidParameter("personalization entries must be finite")
        if x < 0.0:
            raise InvalidParameter("personalization entries must be non-negative")
    s = 0.0
    for x in p:
        s += x
    if s <= 0.0:
        raise InvalidParameter("personalization sum must be > 0")


def personalized_pagerank_checked(graph, config: PageRankConfig, personalization) -> np.ndarray:
    """src/ppr.rs:11-44."""
    config = config or PageRankConfig()
    _check_personalization(graph, config, personalization)
    return personalized_pagerank(graph, config, personalization)


def personalized_pagerank_checked_run(graph, config: PageRankConfig, personalization) -> PageRankRun:
    """src/ppr.rs:77-85 (validated once, solved once)."""
    config = config or PageRankConfig()
    _check_personalization(graph, config, personalization)
    return personalized_pagerank_run(graph, config, personalization)


# ---- ranking helpers used by the parity checks (src/topk.rs) -------------

def top_k(scores: Sequence[float], k: int) -> List[tuple]:
    """src/topk.rs:17-42: the k largest finite, positive scores, descending."""
    if k == 0 or len(scores) == 0:
        return []
    s = np.asarray(scores, dtype=np.float64)
    ok = np.nonzero(np.isfinite(s) & (s > 0.0))[0]
    order = ok[np.argsort(-s[ok], kind="stable")][:k]
    return [(int(i), float(s[i])) for i in order]


def normalize(scores: np.ndarray) -> None:
    """src/topk.rs:54-61 (in place; no-op when the sum is not positive)."""
    total = float(np.sum(scores))
    if total > 0.0:
        scores /= total
