"""Host restatement of the adapter view of a petgraph edge list (test
helper): what neighbors(u) and find_edge(u, v) expose for a
petgraph::Graph<_, f64, Directed> whose raw edges are (src[e], dst[e], w[e])
in edge-index order (src/graph.rs:144-212).  Row u lists the targets of u's
edges newest first; every u -> v entry carries the newest u -> v edge's
weight."""
import numpy as np


def out_csr_from_edges(n, src, dst, w=None):
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    m = src.shape[0]
    eidx = np.arange(m)
    order = np.lexsort((-eidx, src))  # by source, newest edge first
    col = dst[order].astype(np.int32)
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(np.bincount(src, minlength=n))
    if w is None:
        return rp, col, None
    w = np.asarray(w, np.float64)
    newest = {}
    for e in range(m):  # later edges overwrite: the newest u -> v edge wins
        newest[(int(src[e]), int(dst[e]))] = w[e]
    wout = np.array([newest[(int(src[e]), int(dst[e]))] for e in order], np.float64)
    return rp, col, wout
