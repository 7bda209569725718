"""Graph adapters, mirroring graphops' src/graph.rs.

The operators accept anything that behaves like the reference's ``Graph`` /
``WeightedGraph`` traits (src/graph.rs:26-39, 67-72):

* ``node_count()`` and ``neighbors(u)`` (out-neighbours, duplicates allowed),
* optionally ``out_degree(u)`` (default ``len(neighbors(u))``),
* weighted: ``edge_weight(u, v)`` (0.0 when absent).

Three concrete adapters are provided:

* :class:`AdjacencyMatrix` -- ``AdjacencyMatrix(&[Vec<f64>])``
  (src/graph.rs:122-142): edge u->j iff ``M[u][j] > 0.0``, weight ``M[u][j]``.
  Uploaded as the dense matrix; the O(n^2) scan runs on the device.
* :class:`CsrAdjacency` -- an out-adjacency already in CSR arrays (what the
  synthetic generators produce).  Uploaded as is.
* :class:`DiGraph` -- a petgraph-like multigraph (src/graph.rs:144-212):
  ``neighbors`` lists outgoing edges newest first (petgraph's order) and
  ``edge_weight(u, v)`` returns the weight of one u->v edge for every
  parallel duplicate, as ``find_edge`` does.

Any other object with the trait methods is extracted by calling them, exactly
as the reference's own loops call them.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np


class AdjacencyMatrix:
    """Row-major adjacency-matrix adapter (src/graph.rs:122-142)."""

    def __init__(self, matrix: Sequence[Sequence[float]]):
        self.matrix = np.asarray(matrix, dtype=np.float64)
        if self.matrix.size == 0:
            self.matrix = self.matrix.reshape(0, 0)

    def node_count(self) -> int:
        return int(self.matrix.shape[0])

    def neighbors(self, node: int) -> List[int]:
        row = self.matrix[node]
        return [int(j) for j in np.nonzero(row > 0.0)[0]]

    def out_degree(self, node: int) -> int:
        return len(self.neighbors(node))

    def edge_weight(self, source: int, target: int) -> float:
        return float(self.matrix[source][target])


@dataclass
class CsrAdjacency:
    """Out-adjacency in CSR form: row u lists neighbors(u) in order."""
    row_ptr: np.ndarray
    col: np.ndarray
    weight: Optional[np.ndarray] = None

    def node_count(self) -> int:
        return int(len(self.row_ptr) - 1)

    def neighbors(self, node: int) -> List[int]:
        return [int(v) for v in self.col[self.row_ptr[node]:self.row_ptr[node + 1]]]

    def out_degree(self, node: int) -> int:
        return int(self.row_ptr[node + 1] - self.row_ptr[node])

    def edge_weight(self, source: int, target: int) -> float:
        if self.weight is None:
            return 1.0 if target in self.neighbors(source) else 0.0
        lo, hi = self.row_ptr[source], self.row_ptr[source + 1]
        hits = np.nonzero(self.col[lo:hi] == target)[0]
        return float(self.weight[lo + hits[0]]) if hits.size else 0.0

    @classmethod
    def from_generated(cls, g) -> "CsrAdjacency":
        return cls(g.row_ptr, g.col, g.weight)


class DiGraph:
    """A directed multigraph with petgraph's adapter semantics.  It keeps its
    edges in insertion order, like petgraph's edge storage, so the operators
    upload it in bulk (raw_edges -> gops_graph_from_edges, which builds the
    adapter's out-adjacency on the device) instead of walking neighbors()."""

    def __init__(self, n: int = 0):
        self._out: List[List[tuple]] = [[] for _ in range(n)]
        self._src: List[int] = []
        self._dst: List[int] = []
        self._w: List[float] = []

    def add_node(self) -> int:
        self._out.append([])
        return len(self._out) - 1

    def add_edge(self, a: int, b: int, weight: float = 1.0) -> None:
        if not (0 <= a < len(self._out) and 0 <= b < len(self._out)):
            raise IndexError("edge endpoint out of range")
        self._out[a].append((b, float(weight)))
        self._src.append(a)
        self._dst.append(b)
        self._w.append(float(weight))

    def raw_edges(self):
        """(src, dst, weight) arrays in edge-index (insertion) order, as
        petgraph's Graph::raw_edges() exposes them."""
        return (np.asarray(self._src, dtype=np.int32), np.asarray(self._dst, dtype=np.int32),
                np.asarray(self._w, dtype=np.float64))

    def node_count(self) -> int:
        return len(self._out)

    def neighbors(self, node: int) -> List[int]:
        # petgraph walks a node's outgoing edge list from the newest edge
        return [b for b, _ in reversed(self._out[node])]

    def out_degree(self, node: int) -> int:
        return len(self._out[node])

    def edge_weight(self, source: int, target: int) -> float:
        # find_edge returns one matching edge (the first one its walk meets)
        for b, w in reversed(self._out[source]):
            if b == target:
                return w
        return 0.0


def extract(graph, weighted: bool):
    """Out-CSR arrays (row_ptr, col, weights or None) in adapter order, built by
    calling the adapter the way the reference does (src/pagerank.rs:136,226-234)."""
    if isinstance(graph, CsrAdjacency):
        w = None
        if weighted:
            w = (np.ones(len(graph.col)) if graph.weight is None
                 else np.asarray(graph.weight, dtype=np.float64))
        return (np.asarray(graph.row_ptr, dtype=np.int64), np.asarray(graph.col, dtype=np.int32), w)
    n = graph.node_count()
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    cols: List[int] = []
    ws: List[float] = []
    for u in range(n):
        nb = graph.neighbors(u)
        cols.extend(int(v) for v in nb)
        if weighted:
            ws.extend(float(graph.edge_weight(u, int(v))) for v in nb)
        row_ptr[u + 1] = len(cols)
    col = np.asarray(cols, dtype=np.int32)
    return row_ptr, col, (np.asarray(ws, dtype=np.float64) if weighted else None)
