"""gops_graph_upload's input checks (the per-row and per-edge ones run on the
device after the copy): the same statuses and messages as the host checks."""
import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300._native import GopsError

pytestmark = pytest.mark.gpu


def upload(rp, col):
    return go.DeviceGraph.from_csr(np.array(rp, np.int64), np.array(col, np.int32))


def test_bad_neighbor_index():
    for col in ([1, 3], [1, -1]):
        with pytest.raises(GopsError, match="neighbor index out of range"):
            upload([0, 1, 2, 2], col)


def test_decreasing_row_ptr():
    with pytest.raises(GopsError, match="row_ptr must be non-decreasing"):
        upload([0, 2, 1, 2], [1, 2])
    with pytest.raises(GopsError, match="row_ptr must be non-decreasing"):
        upload([0, 1, 2, -1], [1, 2])


def test_valid_after_invalid():
    with pytest.raises(GopsError):
        upload([0, 1, 2, 2], [1, 5])
    g = upload([0, 1, 2, 2], [1, 2])
    s, it, diff, conv = g.pagerank_run(go.PageRankConfig())
    assert conv and abs(s.sum() - 1.0) < 1e-9


def test_weighted_invalid_then_valid():
    """The weights travel on a second stream: a rejected upload still waits
    for that copy before freeing, and the next upload and solve are sound."""
    w = np.array([0.5, 2.0], np.float64)
    with pytest.raises(GopsError, match="neighbor index out of range"):
        go.DeviceGraph.from_csr(np.array([0, 1, 2, 2], np.int64), np.array([1, 7], np.int32), w)
    with pytest.raises(GopsError, match="row_ptr must be non-decreasing"):
        go.DeviceGraph.from_csr(np.array([0, 2, 1, 2], np.int64), np.array([1, 2], np.int32), w)
    g = go.DeviceGraph.from_csr(np.array([0, 1, 2, 2], np.int64), np.array([1, 2], np.int32), w)
    s, it, diff, conv = g.pagerank_weighted_run(go.PageRankConfig())
    assert conv and abs(s.sum() - 1.0) < 1e-9


def _random_multigraph(n, m, seed):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, size=m).astype(np.int32)
    dst = rng.integers(0, n, size=m).astype(np.int32)
    # hubs, parallel edges and self loops
    src[: m // 10] = rng.integers(0, 4, size=m // 10)
    dst[m // 10: m // 5] = src[m // 10: m // 5]
    w = rng.uniform(0.1, 1.0, size=m)
    w[::17] = 0.0
    return src, dst, w


def test_edge_list_upload_matches_the_adapter_walk():
    """gops_graph_from_edges (petgraph's raw edge list, built on the device)
    against the out-adjacency walked on the host (tests/edges_ref.py, equal to
    the adapter walk over neighbors() / find_edge): the same graph, so
    bit-identical weighted, unweighted and personalized solves; and the
    oracle's restatement on the walked arrays within the parity bars."""
    from edges_ref import out_csr_from_edges
    from oracle import port
    n, m = 3000, 60000
    src, dst, w = _random_multigraph(n, m, 5)
    rp, col, ww = out_csr_from_edges(n, src, dst, w)
    bulk = go.DeviceGraph.from_edges(n, src, dst, w)
    walked = go.DeviceGraph.from_csr(rp, col, ww)
    conf = go.PageRankConfig(0.85, 1000, 1e-9)
    a = bulk.pagerank_weighted_run(conf)
    b = walked.pagerank_weighted_run(conf)
    assert np.array_equal(a[0], b[0]) and a[1:] == b[1:]
    ref = port.pagerank_weighted_run(rp, col, ww, 0.85, 1000, 1e-9)
    assert np.abs(a[0] - ref[0]).sum() <= 1e-7 and abs(a[1] - ref[1]) <= 1
    bu = go.DeviceGraph.from_edges(n, src, dst)
    wu = go.DeviceGraph.from_csr(rp, col)
    assert np.array_equal(bu.pagerank_run(conf)[0], wu.pagerank_run(conf)[0])
    p = np.zeros(n)
    p[[3, 77, 1500]] = 1.0
    x = go.personalized_pagerank_run(bu, conf, p)
    y = go.personalized_pagerank_run(wu, conf, p)
    assert np.array_equal(x.scores, y.scores)


def test_edge_list_upload_through_the_digraph_adapter():
    """The operators take a DiGraph through the bulk path; the result equals
    the one from its walked out-adjacency."""
    from graphops_gb300.graph import extract
    g = go.DiGraph(500)
    src, dst, w = _random_multigraph(500, 8000, 9)
    for a, b, x in zip(src, dst, w):
        g.add_edge(int(a), int(b), float(x))
    rp, col, ww = extract(g, weighted=True)
    conf = go.PageRankConfig(0.85, 1000, 1e-9)
    r = go.pagerank_weighted_run(g, conf)
    q = go.pagerank_weighted_run(go.CsrAdjacency(rp, col, ww), conf)
    assert np.array_equal(r.scores, q.scores) and r.iterations == q.iterations


def test_edge_list_checks():
    with pytest.raises(GopsError, match="edge endpoint out of range"):
        go.DeviceGraph.from_edges(4, np.array([0, 1], np.int32), np.array([1, 4], np.int32))
    with pytest.raises(GopsError, match="edge endpoint out of range"):
        go.DeviceGraph.from_edges(4, np.array([-1], np.int32), np.array([1], np.int32))
    e = go.DeviceGraph.from_edges(5, np.zeros(0, np.int32), np.zeros(0, np.int32))
    s, it, _, conv = e.pagerank_run(go.PageRankConfig())
    assert np.allclose(s, 0.2) and conv  # no edges: every node dangling, uniform


def _pair_weight(u, v):
    """A weight per (source, target) pair, so parallel edges carry equal weights
    (the adapter's newest-edge rule then changes nothing); some negative, some
    NaN (both count as 0)."""
    h = (u.astype(np.int64) * 2654435761 + v.astype(np.int64) * 40503) % 1000003
    w = 0.1 + (h % 1000) / 1111.0
    w = np.where(h % 13 == 0, -w, w)
    return np.where(h % 29 == 0, np.nan, w)


def test_large_weighted_upload_matches_the_edge_list_build():
    """gops_graph_upload (weights copied on the second stream while the edge
    sort runs) against gops_graph_from_edges (the same out-adjacency built
    on the device from the raw edge list, weights already there), over 4 M
    edges: rows of 1-7 entries (within one lane's 8 entries of the row-sum
    pass, or across two), 8-256 entries (across lanes and 256-entry tiles),
    257-3,000 entries and a hub row with more than half of the edges (across
    many tiles), rows whose weights are all zero (dangling by weight),
    negative and NaN weights, and rows without edges.  The two
    builds give bit-identical weighted solves, and match the oracle's
    restatement."""
    from oracle import port
    rng = np.random.default_rng(12)
    n = 400_000
    deg = np.zeros(n, np.int64)
    idx = rng.permutation(n)
    deg[idx[:250_000]] = rng.integers(1, 8, 250_000)
    deg[idx[250_000:270_000]] = rng.integers(8, 257, 20_000)
    deg[idx[270_000:270_300]] = rng.integers(257, 3001, 300)
    hub = n // 2
    deg[hub] = 4_200_000
    rp = np.zeros(n + 1, np.int64)
    rp[1:] = np.cumsum(deg)
    m = int(rp[-1])
    assert m >= 1 << 22 and deg[hub] > m // 2
    row = np.repeat(np.arange(n, dtype=np.int64), deg)
    col = rng.integers(0, n, m).astype(np.int32)
    w = _pair_weight(row, col.astype(np.int64))
    for u in idx[1000:1400]:  # light and mid rows whose weights are all zero
        w[rp[u]:rp[u + 1]] = 0.0
    # the raw edge list whose newest-first walk is this CSR: each row reversed
    rev = rp[row] + rp[row + 1] - 1 - np.arange(m, dtype=np.int64)
    src_raw, dst_raw, w_raw = row.astype(np.int32), col[rev], w[rev]
    conf = go.PageRankConfig(0.85, 1000, 1e-9)
    chunked = go.DeviceGraph.from_csr(rp, col, w)
    one = go.DeviceGraph.from_edges(n, src_raw, dst_raw, w_raw)
    a = chunked.pagerank_weighted_run(conf)
    b = one.pagerank_weighted_run(conf)
    assert np.array_equal(a[0], b[0]) and a[1:] == b[1:]
    ref = port.pagerank_weighted_run(rp, col, w, 0.85, 1000, 1e-9)
    assert np.abs(a[0] - ref[0]).sum() <= 1e-7 and abs(a[1] - ref[1]) <= 1
    again = go.DeviceGraph.from_csr(rp, col, w).pagerank_weighted_run(conf)
    assert np.array_equal(a[0], again[0])
