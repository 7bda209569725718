"""Host-side logic that needs no GPU: the C ABI's exports and validators, the
Python mirror's validation messages (the reference's exact strings), the
adapters' semantics and the generators' determinism."""
import ctypes
import hashlib
import os
import re

import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300 import _native, gen
from conftest import ROOT

LIB = os.path.join(ROOT, "graphops_gb300", "libgops.so")
needs_lib = pytest.mark.skipif(not os.path.exists(LIB), reason="libgops.so not built")


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(gops_[a-z0-9_]+)\s*\(", src))
    return names


@needs_lib
def test_library_loads_and_exports_every_declared_symbol():
    lib = ctypes.CDLL(LIB)
    syms = declared_symbols()
    assert len(syms) >= 17
    for s in sorted(syms):
        assert hasattr(lib, s), s
    assert {n for n, _, _ in _native.SIGNATURES} <= syms


@needs_lib
def test_abi_version_and_no_device_status():
    lib = _native.lib()
    assert lib.gops_abi_version() == 1
    import torch
    if not torch.cuda.is_available():
        h = ctypes.c_void_p()
        assert lib.gops_ctx_create(0, ctypes.byref(h)) == _native.GOPS_ERR_NO_DEVICE


def c_validate(cfg):
    lib = _native.lib()
    buf = ctypes.create_string_buffer(256)
    c = _native.Config(cfg.damping, cfg.max_iterations, cfg.tolerance)
    rc = lib.gops_config_validate(ctypes.byref(c), buf, 256)
    return rc, buf.value.decode()


CONFIG_CASES = [
    (go.PageRankConfig(), None),
    (go.PageRankConfig(damping=float("nan")), "damping must be finite"),
    (go.PageRankConfig(damping=float("inf")), "damping must be finite"),
    (go.PageRankConfig(damping=1.5), "damping must be in [0,1]"),
    (go.PageRankConfig(damping=-0.1), "damping must be in [0,1]"),
    (go.PageRankConfig(max_iterations=0), "max_iterations must be > 0"),
    (go.PageRankConfig(tolerance=0.0), "tolerance must be finite and > 0"),
    (go.PageRankConfig(tolerance=float("nan")), "tolerance must be finite and > 0"),
    (go.PageRankConfig(damping=0.0), None),
    (go.PageRankConfig(damping=1.0), None),
]


@pytest.mark.parametrize("cfg,msg", CONFIG_CASES)
def test_config_validate_messages(cfg, msg):
    """src/pagerank.rs:63-85: Python mirror and C ABI give the same message."""
    if msg is None:
        cfg.validate()
    else:
        with pytest.raises(go.InvalidParameter) as e:
            cfg.validate()
        assert e.value.msg == msg
        assert str(e.value) == f"invalid parameter: {msg}"
    if os.path.exists(LIB):
        rc, m = c_validate(cfg)
        assert (rc == 0) == (msg is None)
        if msg:
            assert m == msg


def test_checked_wrappers_validate_before_any_device_work():
    adj = go.AdjacencyMatrix([[0.0, 1.0], [0.0, 0.0]])
    with pytest.raises(go.InvalidParameter, match="personalization length"):
        go.personalized_pagerank_checked(adj, go.PageRankConfig(), [1.0])       # src/ppr.rs:163-171
    with pytest.raises(go.InvalidParameter, match="sum"):
        go.personalized_pagerank_checked(adj, go.PageRankConfig(), [0.0, 0.0])  # src/ppr.rs:173-181
    with pytest.raises(go.InvalidParameter, match="non-negative"):
        go.personalized_pagerank_checked(adj, go.PageRankConfig(), [1.0, -1.0])
    with pytest.raises(go.InvalidParameter, match="finite"):
        go.personalized_pagerank_checked(adj, go.PageRankConfig(), [1.0, float("nan")])
    with pytest.raises(go.InvalidParameter, match="max_iterations"):
        go.pagerank_checked(adj, go.PageRankConfig(max_iterations=0))


@pytest.mark.parametrize("n,u,v", [(2, 0, 1), (5, 3, 3), (9, 8, 2)])
def test_weighted_checked_rejects_negative(n, u, v):
    """src/pagerank.rs:397-424, with the reference's TestWeighted adapter."""
    class TestWeighted:
        def __init__(self, neighbors, w):
            self.nb, self.w = neighbors, w
        def node_count(self):
            return len(self.nb)
        def neighbors(self, node):
            return list(self.nb[node])
        def edge_weight(self, s, t):
            return self.w[s][t]
    u = u % n
    v = v % n
    if v == u:
        v = (v + 1) % n
    nb = [[] for _ in range(n)]
    w = [[0.0] * n for _ in range(n)]
    nb[u].append(v)
    w[u][v] = -1.0
    with pytest.raises(go.InvalidParameter, match="non-negative"):
        go.pagerank_weighted_checked(TestWeighted(nb, w), go.PageRankConfig())
    w[u][v] = float("inf")
    with pytest.raises(go.InvalidParameter, match="finite"):
        go.pagerank_weighted_checked(TestWeighted(nb, w), go.PageRankConfig())


@needs_lib
def test_c_abi_weight_and_personalization_validators():
    lib = _native.lib()
    buf = ctypes.create_string_buffer(256)
    w = np.array([1.0, -2.0])
    assert lib.gops_weights_validate(2, _native.ptr(w), buf, 256) == 1
    assert buf.value.decode() == "edge weights must be non-negative"
    w = np.array([1.0, np.inf])
    assert lib.gops_weights_validate(2, _native.ptr(w), buf, 256) == 1
    assert buf.value.decode() == "edge weights must be finite"
    p = np.array([1.0])
    assert lib.gops_personalization_validate(2, 1, _native.ptr(p), buf, 256) == 1
    assert buf.value.decode() == "personalization length must equal node_count (len=1 node_count=2)"
    p = np.zeros(2)
    assert lib.gops_personalization_validate(2, 2, _native.ptr(p), buf, 256) == 1
    assert buf.value.decode() == "personalization sum must be > 0"
    p = np.array([0.5, 0.5])
    assert lib.gops_personalization_validate(2, 2, _native.ptr(p), buf, 256) == 0


def test_adjacency_matrix_adapter():
    """src/graph.rs:107-121 doctest and the w > 0.0 rule."""
    m = go.AdjacencyMatrix([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]])
    assert m.node_count() == 3 and m.neighbors(0) == [1]
    m = go.AdjacencyMatrix([[0.0, -1.0, float("nan"), 2.0]] * 4)
    assert m.neighbors(0) == [3] and m.edge_weight(0, 1) == -1.0


def test_petgraph_like_adapter_order_and_find_edge():
    g = go.DiGraph(3)
    g.add_edge(0, 1, 1.0)
    g.add_edge(0, 2, 5.0)
    g.add_edge(0, 1, 7.0)
    assert g.neighbors(0) == [1, 2, 1]          # newest first, duplicates kept
    assert g.edge_weight(0, 1) == 7.0           # one edge's weight for every duplicate
    rp, col, w = go.graph.extract(g, weighted=True)
    assert rp.tolist() == [0, 3, 3, 3] and col.tolist() == [1, 2, 1] and w.tolist() == [7.0, 5.0, 7.0]


def _digest(g):
    h = hashlib.sha256()
    h.update(g.row_ptr.tobytes()); h.update(g.col.tobytes())
    if g.weight is not None:
        h.update(g.weight.tobytes())
    return h.hexdigest()[:16]


# Digests of small generated graphs: the generators are integer-threshold,
# counter-based and built without FMA contraction, so these hold on x86-64
# and AArch64 alike and for any thread count.
GEN_DIGESTS = {
    "er": "f911f03d2ccb4bda",
    "rmat": "1d59e26ff5906fd7",
    "sbm": "2fcbf6447c8fa523",
}


def test_generators_are_deterministic_across_thread_counts():
    a = gen.rmat(12, 16, weighted=True, seed=11, threads=1)
    b = gen.rmat(12, 16, weighted=True, seed=11, threads=7)
    assert _digest(a) == _digest(b)
    s1 = gen.sbm(3000, 8, seed=3, threads=1)
    s2 = gen.sbm(3000, 8, seed=3, threads=5)
    assert _digest(s1) == _digest(s2) and np.array_equal(s1.block, s2.block)


def test_generator_shapes():
    g = gen.erdos_renyi(2000, 0.005, 0.01, seed=0)
    deg = g.out_degree()
    assert g.n == 2000 and (deg == 0).sum() >= 20
    assert 15000 < g.m < 25000
    src = np.repeat(np.arange(g.n), deg)
    assert not np.any(src == g.col)
    r = gen.rmat(14, 16, weighted=True, seed=1)
    src = np.repeat(np.arange(r.n), r.out_degree())
    key = src * r.n + r.col
    assert np.all(np.diff(key) > 0)             # sorted, no duplicates
    assert not np.any(src == r.col)             # no self loops
    assert r.weight.min() >= 0.1 and r.weight.max() < 1.0
    s = gen.sbm(5000, 64, seed=2)
    assert s.block.min() == 0 and s.block.max() == 63
    sizes = np.bincount(s.block)
    assert sizes[0] > sizes[-1] and sizes.sum() == 5000
    sp, si = gen.seed_sets(r, 50, 1, 64, seed=9)
    lens = np.diff(sp)
    assert lens.min() >= 1 and lens.max() <= 64
    for i in range(50):
        assert len(set(si[sp[i]:sp[i + 1]].tolist())) == lens[i]


def test_generator_digests():
    got = {
        "er": _digest(gen.erdos_renyi(300, 0.02, 0.01, seed=1)),
        "rmat": _digest(gen.rmat(10, 8, weighted=True, seed=2)),
        "sbm": _digest(gen.sbm(1000, 8, seed=3)),
    }
    assert got == GEN_DIGESTS, got


def test_digraph_raw_edges_restate_the_adapter_walk():
    """The bulk path's expected out-adjacency (tests/edges_ref.py, what the
    device builds from raw_edges) equals the adapter walk over neighbors()
    and edge_weight() on a multigraph with parallel edges and self loops."""
    from edges_ref import out_csr_from_edges
    from graphops_gb300.graph import extract
    rng = np.random.default_rng(11)
    g = go.DiGraph(40)
    for _ in range(400):
        a, b = rng.integers(0, 40, size=2)
        g.add_edge(int(a), int(b), float(rng.choice([0.0, 0.5, 1.5, rng.random()])))
    for _ in range(30):  # parallel edges with their own weights
        a, b = rng.integers(0, 5, size=2)
        g.add_edge(int(a), int(b), float(rng.random()))
    src, dst, w = g.raw_edges()
    rp, col, ww = out_csr_from_edges(g.node_count(), src, dst, w)
    rp2, col2, ww2 = extract(g, weighted=True)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2) and np.array_equal(ww, ww2)
    with pytest.raises(IndexError):
        g.add_edge(0, 40)
