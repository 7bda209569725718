"""Katz and eigenvector centrality on the GPU (gops_katz_run,
gops_eigenvector_run) against the C restatement of the reference loops:
FP64 on both sides, summation order differs, so scores agree to ~1e-15
relative and the iteration counts exactly (a step whose L1 lands within a
few ulps of the tolerance could differ by one; none does here)."""
import math

import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300 import gen
from oracle import port

pytestmark = pytest.mark.gpu
REL = 1e-12


def csr(adj):
    rp = np.zeros(len(adj) + 1, dtype=np.int64)
    for i, r in enumerate(adj):
        rp[i + 1] = rp[i] + len(r)
    col = np.array([v for r in adj for v in r], dtype=np.int32)
    return rp, col


def rel_l1(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


SMALL = [
    [[1], [0, 2], [1, 3], [2]],
    [[1, 2], [0, 2], [0, 1]],
    [[1, 2, 3, 4], [0], [0], [0], [0]],
    [[1, 2, 3], [0, 2], [0, 1, 3], [0, 2]],
    [[], [], []],
    [[0, 1, 1], [2], []],            # self loop, duplicate edge, dangling node
]


@pytest.mark.parametrize("adj", SMALL)
def test_small_graphs_match_oracle(adj):
    rp, col = csr(adj)
    dg = go.DeviceGraph.from_csr(rp, col)
    for kw in ({}, {"alpha": 0.3, "beta": 2.0, "tolerance": 1e-10}):
        cfg = go.KatzConfig(**kw)
        r = go.katz_centrality_run(dg, cfg)
        s, it, diff, conv = port.katz_run(rp, col, cfg.alpha, cfg.beta, cfg.max_iterations, cfg.tolerance)
        assert r.iterations == it and r.converged == conv
        assert rel_l1(r.scores, s) <= REL
    r = go.eigenvector_centrality_run(dg, 100, 1e-8)
    s, it, diff, conv = port.eigenvector_run(rp, col, 100, 1e-8)
    assert r.iterations == it and r.converged == conv
    assert rel_l1(r.scores, s) <= REL


@pytest.mark.parametrize("scale", [10, 14])
def test_rmat_katz_converging_and_diverging(scale):
    g = gen.rmat(scale, 16, seed=scale)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    indeg = np.bincount(g.col, minlength=g.n)
    a = 0.5 / max(int(indeg.max()), 1)   # below 1/rho(A): converges
    for alpha, tol, it_max in ((a, 1e-6, 1000), (0.1, 1e-6, 30)):   # 0.1: grows without bound
        r = go.katz_centrality_run(dg, go.KatzConfig(alpha, 1.0, it_max, tol))
        s, it, diff, conv = port.katz_run(g.row_ptr, g.col, alpha, 1.0, it_max, tol)
        assert r.iterations == it and r.converged == conv
        assert rel_l1(r.scores, s) <= REL
        # the step norm sums differences of nearly equal values: its error
        # scales with the vector's mass, not with the step
        assert abs(r.diff_l1 - diff) <= 1e-13 * np.abs(s).sum()


@pytest.mark.parametrize("seed", [0, 1])
def test_eigenvector_directed_and_symmetric(seed):
    g = gen.erdos_renyi(3000, 0.004, 0.02, seed=seed)
    for symmetric in (False, True):
        rp, col = g.row_ptr, g.col
        if symmetric:   # both directions of every edge
            src = np.repeat(np.arange(g.n), np.diff(g.row_ptr))
            u = np.concatenate([src, g.col]); v = np.concatenate([g.col, src])
            o = np.lexsort((v, u)); u, v = u[o], v[o]
            rp = np.zeros(g.n + 1, np.int64); np.add.at(rp, u + 1, 1); rp = np.cumsum(rp)
            col = v.astype(np.int32)
        dg = go.DeviceGraph.from_csr(rp, col)
        r = go.eigenvector_centrality_run(dg, 300, 1e-9)
        s, it, diff, conv = port.eigenvector_run(rp, col, 300, 1e-9)
        assert r.iterations == it and r.converged == conv
        assert rel_l1(r.scores, s) <= REL
        assert abs(np.sqrt((r.scores ** 2).sum()) - 1.0) < 1e-12


def test_adapters_dense_and_weighted_ignore_weights():
    rng = np.random.default_rng(3)
    M = (rng.random((40, 40)) < 0.1) * rng.random((40, 40))
    a = go.eigenvector_centrality(go.AdjacencyMatrix(M))
    rp, col = port.dense_to_csr(M)[:2]
    s, *_ = port.eigenvector_run(rp, col)
    assert rel_l1(a, s) <= REL
    g = gen.rmat(9, 8, weighted=True, seed=2)
    dw = go.DeviceGraph.from_csr(g.row_ptr, g.col, g.weight.astype(np.float64))
    du = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    k1 = go.katz_centrality(dw, go.KatzConfig(alpha=0.01))
    k2 = go.katz_centrality(du, go.KatzConfig(alpha=0.01))
    assert np.array_equal(k1, k2)


def test_edge_runs():
    rp, col = csr([[1], [0]])
    dg = go.DeviceGraph.from_csr(rp, col)
    r = go.katz_centrality_run(dg, go.KatzConfig(max_iterations=0))
    assert r.iterations == 0 and math.isinf(r.diff_l1) and not r.converged and (r.scores == 1.0).all()
    r = go.eigenvector_centrality_run(dg, 0, 1e-6)
    assert r.iterations == 0 and r.diff_l1 == 0.0 and not r.converged
    assert np.allclose(r.scores, 1 / math.sqrt(2))
    e = go.eigenvector_centrality_run(go.CsrAdjacency(np.zeros(1, np.int64), np.zeros(0, np.int32)))
    assert len(e.scores) == 0 and e.converged


@pytest.mark.parametrize("adj", SMALL + [[[1, 2, 3, 4], [], [], [], []]])
def test_hits_small_match_oracle(adj):
    rp, col = csr(adj)
    dg = go.DeviceGraph.from_csr(rp, col)
    hub, auth, it, d, conv = dg.hits_run(100, 1e-10)
    rh, ra, rit, rd, rconv = port.hits_run(rp, col, 100, 1e-10)
    assert it == rit and conv == rconv
    assert rel_l1(hub, rh) <= REL and rel_l1(auth, ra) <= REL


@pytest.mark.parametrize("scale", [10, 13])
def test_hits_rmat_matches_oracle(scale):
    g = gen.rmat(scale, 8, seed=scale + 5)
    hub, auth = go.hits(go.CsrAdjacency(g.row_ptr, g.col), 200, 1e-9)
    rh, ra, rit, rd, rconv = port.hits_run(g.row_ptr, g.col, 200, 1e-9)
    assert rel_l1(hub, rh) <= 1e-10 and rel_l1(auth, ra) <= 1e-10
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    _, _, it, d, conv = dg.hits_run(200, 1e-9)
    assert abs(it - rit) <= 1 and conv == rconv


def test_long_rows_summed_in_chunks_match_oracle():
    """Hub rows above 2,048 edges are summed in 8,192-edge chunks (a block
    each) and the chunk sums added in order: Katz, eigenvector centrality
    and HITS on a graph whose hubs have ~20,000 in- and out-edges (several
    chunks, the last partial) against the oracle, and R-MAT scale 17 (hubs of
    a few thousand edges)."""
    rng = np.random.default_rng(7)
    n = 20000
    src = [np.zeros(n - 1, np.int64), np.arange(1, n), rng.integers(0, n, 60000)]
    dst = [np.arange(1, n), np.full(n - 1, 1), rng.integers(0, n, 60000)]
    u = np.concatenate(src)
    v = np.concatenate(dst)
    o = np.argsort(u, kind="stable")
    u, v = u[o], v[o]
    rp = np.zeros(n + 1, np.int64)
    np.add.at(rp, u + 1, 1)
    rp = np.cumsum(rp)
    col = v.astype(np.int32)
    assert np.diff(rp).max() > 2 * 8192 and np.bincount(col, minlength=n).max() > 2 * 8192
    g = gen.rmat(17, 16, seed=17)
    for rp_, col_ in ((rp, col), (g.row_ptr, g.col)):
        dg = go.DeviceGraph.from_csr(rp_, col_)
        indeg = np.bincount(col_, minlength=len(rp_) - 1)
        alpha = 0.5 / max(int(indeg.max()), 1)
        r = go.katz_centrality_run(dg, go.KatzConfig(alpha, 1.0, 1000, 1e-9))
        s, it, diff, conv = port.katz_run(rp_, col_, alpha, 1.0, 1000, 1e-9)
        assert r.iterations == it and r.converged == conv
        assert rel_l1(r.scores, s) <= REL
        r = go.eigenvector_centrality_run(dg, 200, 1e-9)
        s, it, diff, conv = port.eigenvector_run(rp_, col_, 200, 1e-9)
        assert r.iterations == it and r.converged == conv
        assert rel_l1(r.scores, s) <= REL
        hub, auth, it, d, conv = dg.hits_run(200, 1e-9)
        rh, ra, rit, rd, rconv = port.hits_run(rp_, col_, 200, 1e-9)
        assert abs(it - rit) <= 1 and conv == rconv
        assert rel_l1(hub, rh) <= 1e-10 and rel_l1(auth, ra) <= 1e-10
