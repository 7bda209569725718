"""Pure-Python restatement of graphops' PageRank / PPR power iteration.

TEST INFRASTRUCTURE ONLY (the oracle).  Used on small graphs to cross-check
the C restatement in ``pagerank_port.c`` bit for bit, and to generate the
golden fixtures under ``tests/golden``.  The product never imports this.

Each function follows the reference line by line, in FP64 (Python floats),
with the same loop and summation order, so results are bitwise equal to the
reference's own arithmetic on the same adapter order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Sequence


@dataclass
class Run:
    scores: List[float]
    iterations: int
    diff_l1: float
    converged: bool


def _rust_max0(w: float) -> float:
    # f64::max(w, 0.0): NaN yields the other argument.
    if math.isnan(w):
        return 0.0
    return w if w > 0.0 else 0.0


def dense_neighbors(M: Sequence[Sequence[float]]) -> List[List[int]]:
    """AdjacencyMatrix::neighbors (src/graph.rs:128-135): w > 0.0, ascending j."""
    return [[j for j, w in enumerate(row) if w > 0.0] for row in M]


def pagerank_run(neighbors: Sequence[Sequence[int]], damping: float,
                 max_iterations: int, tolerance: float) -> Run:
    """src/pagerank.rs:122-187."""
    n = len(neighbors)
    if n == 0:
        return Run([], 0, 0.0, True)
    n_f = float(n)
    scores = [1.0 / n_f] * n
    new = [0.0] * n
    deg = [len(nb) for nb in neighbors]
    iters, last, conv = 0, math.inf, False
    for _ in range(max_iterations):
        iters += 1
        dsum = 0.0
        for i in range(n):
            if deg[i] == 0:
                dsum += scores[i]
        fill = (1.0 - damping) / n_f + damping * dsum / n_f
        new = [fill] * n
        for u in range(n):
            if deg[u] > 0:
                share = damping * scores[u] / float(deg[u])
                for v in neighbors[u]:
                    new[v] += share
        diff = 0.0
        for a, b in zip(scores, new):
            diff += abs(a - b)
        last = diff
        scores, new = new, scores
        if diff < tolerance:
            conv = True
            break
    return Run(scores, iters, last, conv)


def pagerank_weighted_run(neighbors: Sequence[Sequence[int]],
                          weights: Sequence[Sequence[float]], damping: float,
                          max_iterations: int, tolerance: float) -> Run:
    """src/pagerank.rs:210-289.  weights[u][k] = edge_weight(u, neighbors[u][k])."""
    n = len(neighbors)
    if n == 0:
        return Run([], 0, 0.0, True)
    n_f = float(n)
    scores = [1.0 / n_f] * n
    ws = []
    for u in range(n):
        s = 0.0
        for w in weights[u]:
            s += _rust_max0(w)
        ws.append(s)
    iters, last, conv = 0, math.inf, False
    for _ in range(max_iterations):
        iters += 1
        dsum = 0.0
        for i in range(n):
            if ws[i] == 0.0:
                dsum += scores[i]
        fill = (1.0 - damping) / n_f + damping * dsum / n_f
        new = [fill] * n
        for u in range(n):
            if ws[u] > 0.0:
                for v, w in zip(neighbors[u], weights[u]):
                    w = _rust_max0(w)
                    if w > 0.0:
                        new[v] += damping * scores[u] * (w / ws[u])
        diff = 0.0
        for a, b in zip(scores, new):
            diff += abs(a - b)
        last = diff
        scores = new
        if diff < tolerance:
            conv = True
            break
    return Run(scores, iters, last, conv)


def personalized_pagerank_run(neighbors: Sequence[Sequence[int]],
                              personalization: Sequence[float], damping: float,
                              max_iterations: int, tolerance: float) -> Run:
    """src/ppr.rs:90-156 (unweighted; dangling mass returns to p)."""
    n = len(neighbors)
    if n == 0:
        return Run([], 0, 0.0, True)
    psum = 0.0
    for x in personalization:
        psum += x
    if psum > 0.0:
        p = [x / psum for x in personalization]
    else:
        p = [1.0 / float(n)] * n
    scores = list(p)
    deg = [len(nb) for nb in neighbors]
    iters, last, conv = 0, math.inf, False
    for _ in range(max_iterations):
        iters += 1
        dsum = 0.0
        for i in range(n):
            if deg[i] == 0:
                dsum += scores[i]
        new = [(1.0 - damping) * p[i] + damping * dsum * p[i] for i in range(n)]
        for u in range(n):
            if deg[u] > 0:
                share = damping * scores[u] / float(deg[u])
                for v in neighbors[u]:
                    new[v] += share
        diff = 0.0
        for a, b in zip(scores, new):
            diff += abs(a - b)
        last = diff
        scores = new
        if diff < tolerance:
            conv = True
            break
    return Run(scores, iters, last, conv)
