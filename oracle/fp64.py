"""Independent FP64 oracle for PageRank / personalized PageRank fixed points.

TEST INFRASTRUCTURE ONLY.  It does not follow the reference's loop; it solves
for the exact fixed point of the same Markov chain, so "error vs the FP64
oracle" can be reported independently of any iteration order:

  plain / weighted (src/pagerank.rs:122-289):
      x = (1-d)/n * 1 + d * (P^T x + (sum_{u dangling} x_u) / n * 1)
  personalized (src/ppr.rs:90-156):
      x = (1-d) p + d * (sum_{u dangling} x_u) p + d * P^T x

P[u, v] = (#edges u->v) / deg(u) unweighted, or sum of max(w, 0) over u->v
divided by sum over u's out-edges of max(w, 0) weighted; a node is dangling
when deg == 0 (unweighted) or its weight sum == 0 (weighted).

Small n: dense LU solve.  Larger n: FP64 power iteration with the exact
dangling term until the step is below 1e-15 in L1.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def transition(n, row_ptr, col, weights=None):
    """Returns (P as CSR n x n float64, dangling mask)."""
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    deg = np.diff(row_ptr)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    if weights is None:
        vals = np.ones(col.shape[0], dtype=np.float64)
    else:
        w = np.asarray(weights, dtype=np.float64)
        vals = np.where(np.isnan(w), 0.0, np.maximum(w, 0.0))
    rows_sum = np.bincount(src, weights=vals, minlength=n) if n else np.zeros(0)
    dangling = rows_sum == 0.0
    scale = np.zeros(n)
    scale[~dangling] = 1.0 / rows_sum[~dangling]
    P = sp.csr_matrix((vals * scale[src], (src, col)), shape=(n, n))
    return P, dangling


def fixed_point(n, row_ptr, col, damping, weights=None, personalization=None,
                dense_limit=3000, tol=1e-15, max_iter=100000):
    """Exact (to ~1e-15) FP64 fixed point of the reference's iteration."""
    if n == 0:
        return np.zeros(0)
    P, dangling = transition(n, row_ptr, col, weights)
    PT = P.T.tocsr()
    if personalization is None:
        b = np.full(n, (1.0 - damping) / n)
        r = np.full(n, 1.0 / n)          # dangling mass spreads uniformly
    else:
        p = np.asarray(personalization, dtype=np.float64)
        s = p.sum()
        p = p / s if s > 0 else np.full(n, 1.0 / n)
        b = (1.0 - damping) * p
        r = p                            # dangling mass returns to p
    if n <= dense_limit:
        A = np.eye(n) - damping * PT.toarray() - damping * np.outer(r, dangling.astype(np.float64))
        return np.linalg.solve(A, b)
    x = r.copy() if personalization is not None else np.full(n, 1.0 / n)
    for _ in range(max_iter):
        nx = b + damping * (PT @ x) + damping * x[dangling].sum() * r
        step = np.abs(nx - x).sum()
        x = nx
        if step < tol:
            break
    return x
