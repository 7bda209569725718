"""Parity at the benchmark sizes: the GPU results of the benchmarked
workloads against the oracle's C restatement of the reference on the same
inputs, plus size-independent properties of the same results.

Bars (the reference's correctness contract for this path):
  * L1(gpu, restatement) <= 1e-6 per result (the parity bar), and the
    measured value is asserted below the tighter bar written beside each case;
  * identical top-100 order (ties within 1e-15 relative count as equal; the
    batched path's FP32 score blocks cannot order entries more finely than
    their own error, so there two entries may swap only when their
    reference scores differ by less than twice the result's largest error);
  * iteration counts within +-1 of the restatement's for the plain path
    (a learned warm start changes where the iteration starts, so its count
    is compared with the plain path's instead).

Cases:
  * weighted PageRank on R-MAT scale 22 (the bench workload), tol 1e-8,
    against pagerank_weighted_run (src/pagerank.rs:210-289), the serial
    restatement, ~10-20 s on one host core;
  * weighted PageRank on R-MAT scale 25 (the stress workload), tol 1e-8,
    against the restatement's all-cores pull form (FP64; it equals the serial
    form within 1e-12 in L1 with the same step count, tests/test_oracle.py),
    because the serial form takes minutes at 0.53 G edges;
  * batched PPR on R-MAT scale 20, the bench's 1,024 seed sets, 64 of them
    against personalized_pagerank_run (src/ppr.rs:90-156);
  * plain and learned batched PPR on the block-model graph (n = 500,000), the
    bench's held-out sets, 64 of them against personalized_pagerank_run;
  * what the trained network gains: the same learned pipeline with the
    network switched off (w = 1 for every node: same push, clusters and
    least-squares coupling), against the trained network and a cold start.

Size-independent properties (on the same results): non-negative, sums to 1,
a fixed point of the FP64 map to 1e-7 (R-MAT 22), and linearity of the
personalized solution in the personalization (R-MAT 20).
"""
import os

import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300 import gen
from conftest import fp32_tie, sample_sets, top_order_matches
from oracle import port

pytestmark = pytest.mark.gpu
sp_mod = pytest.importorskip("scipy.sparse")

L1_PARITY = 1e-6
THREADS = max(1, os.cpu_count() or 1)


def transition(g, weights):
    """Column-stochastic map of the reference (src/pagerank.rs:210-289) as a
    sparse FP64 matrix A with A[v, u] = max(w,0)/ws(u), and the dangling mask."""
    n = g.n
    src = np.repeat(np.arange(n), np.diff(g.row_ptr))
    if weights is None:
        w = np.ones(g.col.shape[0])
    else:
        w = np.maximum(weights.astype(np.float64), 0.0)
    ws = np.bincount(src, weights=w, minlength=n)
    keep = w > 0
    vals = w[keep] / ws[src[keep]]
    A = sp_mod.csr_matrix((vals, (g.col[keep], src[keep])), shape=(n, n))
    return A, ws == 0.0


# ---------------------------------------------------------------- R-MAT 22

@pytest.fixture(scope="module")
def rmat22():
    g = gen.rmat(22, 16, 0.57, 0.19, 0.19, weighted=True, wlo=0.1, whi=1.0, seed=22)
    r = go.pagerank_weighted_run(go.CsrAdjacency(g.row_ptr, g.col, g.weight), go.PageRankConfig(0.85, 1000, 1e-8))
    return g, r


def test_weighted_pagerank_rmat22_matches_restatement(rmat22):
    g, r = rmat22
    ref, its, diff, conv = port.pagerank_weighted_run(g.row_ptr, g.col, g.weight.astype(np.float64), 0.85, 1000,
                                                      1e-8)
    l1 = float(np.abs(r.scores - ref).sum())
    info = (l1, r.iterations, its, r.diff_l1, diff)
    assert r.converged and conv, info
    assert l1 <= 1e-7, info  # parity bar 1e-6; FP32 ranks with a double-float first phase reach ~1e-8
    assert abs(r.iterations - its) <= 1, info
    assert top_order_matches(r.scores, ref), info


def test_weighted_pagerank_rmat22_fixed_point(rmat22):
    g, r = rmat22
    tol = 1e-8
    x = r.scores
    assert r.converged and r.diff_l1 < tol
    assert x.min() >= 0.0
    assert abs(x.sum() - 1.0) < 1e-6
    A, dang = transition(g, g.weight)
    n = g.n
    fx = (1.0 - 0.85) / n + 0.85 * x[dang].sum() / n + 0.85 * (A @ x)
    # the last step moved less than tol; one more application moves x by at
    # most 0.85 of that, plus FP32 rounding of the stored transition weights
    assert np.abs(fx - x).sum() < 1e-7


# ---------------------------------------------------------------- R-MAT 25

def test_weighted_pagerank_rmat25_matches_restatement():
    g = gen.rmat(25, 16, 0.57, 0.19, 0.19, weighted=True, wlo=0.1, whi=1.0, seed=25)
    r = go.pagerank_weighted_run(go.CsrAdjacency(g.row_ptr, g.col, g.weight), go.PageRankConfig(0.85, 1000, 1e-8))
    ref, its, diff, conv, _ = port.pagerank_weighted_run_mt(g.row_ptr, g.col, g.weight.astype(np.float64), 0.85,
                                                            1000, 1e-8, threads=THREADS)
    l1 = float(np.abs(r.scores - ref).sum())
    info = (l1, r.iterations, its, r.diff_l1, diff)
    assert r.converged and conv, info
    assert l1 <= 1e-7, info
    assert abs(r.iterations - its) <= 1, info
    assert top_order_matches(r.scores, ref), info
    assert r.scores.min() >= 0.0 and abs(r.scores.sum() - 1.0) < 1e-6


# ------------------------------------------------------- batched, R-MAT 20

@pytest.fixture(scope="module")
def rmat20_batch():
    g = gen.rmat(20, 16, seed=20)
    sp, si = gen.seed_sets(g, 1024, 1, 64, seed=7)  # the bench's sets (rank 0)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    r = go.ppr_batch(dg, go.PageRankConfig(0.85, 1000, 1e-7), sp, si)
    return g, sp, si, dg, r


def test_batched_ppr_rmat20_matches_restatement(rmat20_batch):
    g, sp, si, _, r = rmat20_batch
    assert r.converged.all()
    idx = np.arange(0, len(sp) - 1, 16)
    sp2, si2 = sample_sets(sp, si, idx)
    ref, its = port.ppr_many(g.row_ptr, g.col, sp2, si2, 0.85, 1000, 1e-7, threads=THREADS)
    x = r.scores[idx].astype(np.float64)
    l1 = np.abs(x - ref).sum(axis=1)
    assert l1.max() <= 1e-7, (l1.max(), int(l1.argmax()))  # parity bar 1e-6
    assert np.abs(r.iterations[idx] - its.astype(np.int64)).max() <= 1
    for q in range(len(idx)):
        assert top_order_matches(x[q], ref[q], tie=fp32_tie(x[q], ref[q])), q


def test_batched_ppr_rmat20_linearity(rmat20_batch):
    g, _, _, dg, _ = rmat20_batch
    rng = np.random.default_rng(5)
    deg = np.diff(g.row_ptr).astype(np.float64)
    prob = deg / deg.sum()
    sets = []
    for _ in range(32):
        k1, k2 = rng.integers(1, 33, size=2)
        nodes = rng.choice(g.n, size=k1 + k2, replace=False, p=prob)
        s1, s2 = np.sort(nodes[:k1]), np.sort(nodes[k1:])
        sets += [s1, s2, np.sort(np.concatenate([s1, s2]))]
    sp = np.zeros(len(sets) + 1, np.int64)
    sp[1:] = np.cumsum([len(s) for s in sets])
    si = np.concatenate(sets).astype(np.int32)
    r = go.ppr_batch(dg, go.PageRankConfig(0.85, 1000, 1e-7), sp, si)
    assert r.converged.all()
    x = r.scores.astype(np.float64)
    assert x.min() >= 0.0
    assert np.abs(x.sum(axis=1) - 1.0).max() < 1e-6
    dang = deg == 0
    c = (1.0 - 0.85) + 0.85 * x[:, dang].sum(axis=1)
    for q in range(32):
        a, b, u = 3 * q, 3 * q + 1, 3 * q + 2
        na, nb = len(sets[a]), len(sets[b])
        mix = (na * x[a] / c[a] + nb * x[b] / c[b]) / (na + nb)
        # each column is within ~1e-7 of its exact vector (tolerance 1e-7 per set)
        assert np.abs(x[u] / c[u] - mix).sum() < 1e-6, q


# ------------------------------------------------ learned, block model 500k

@pytest.fixture(scope="module")
def sbm_model():
    from graphops_gb300 import warm
    g = gen.sbm(500000, 64, 1.2, 16.0, 4.0, seed=3)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    model = warm.WarmStart(dg, g.row_ptr, g.col, warm.default_config(chunk=512, clusters=72))
    sp_t, si_t = gen.seed_sets(g, 8192, 1, 32, seed=31)
    model.train(conf, sp_t, si_t)
    sp, si = gen.seed_sets(g, 4096, 1, 32, seed=77)  # the bench's held-out sets (rank 0)
    return g, conf, dg, model, sp, si


def test_plain_and_learned_sbm500k_match_restatement(sbm_model):
    g, conf, dg, model, sp, si = sbm_model
    idx = np.arange(0, len(sp) - 1, 64)
    sp2, si2 = sample_sets(sp, si, idx)
    ref, its = port.ppr_many(g.row_ptr, g.col, sp2, si2, 0.85, 1000, 1e-7, threads=THREADS)
    pr = go.ppr_batch(dg, conf, sp2, si2)
    lr = model.ppr_batch(conf, sp2, si2, scores=True)
    assert pr.converged.all() and lr.converged.all()
    for name, x in (("plain", pr.scores), ("learned", lr.scores)):
        x = x.astype(np.float64)
        l1 = np.abs(x - ref).sum(axis=1)
        # each result is within d/(1-d) tol of the fixed point, like the restatement's own
        assert l1.max() <= L1_PARITY, (name, l1.max(), int(l1.argmax()))
        for q in range(len(idx)):
            assert top_order_matches(x[q], ref[q], tie=fp32_tie(x[q], ref[q])), (name, q)
    assert np.abs(pr.iterations - its.astype(np.int64)).max() <= 1
    assert (lr.iterations < pr.iterations).mean() > 0.9


def test_trained_network_beats_network_off_and_cold(sbm_model):
    """The trained network against the same pipeline without it: every node's
    weight w = 1 (w3 = b3 = 0), so the tail mass of each cluster is spread
    evenly over the cluster, with the same exact push, clusters and
    least-squares cluster coupling; and against the cold start from s."""
    from graphops_gb300 import warm
    g, conf, dg, model, sp, si = sbm_model
    idx = np.arange(0, len(sp) - 1, 8)  # 512 held-out sets
    sp2, si2 = sample_sets(sp, si, idx)
    trained = model.ppr_batch(conf, sp2, si2, scores=True)
    params = model.get(warm.PARAMS)
    off = params.copy()
    off[warm.P_W3:warm.P_B3 + 1] = 0.0
    model.set(warm.PARAMS, off)
    try:
        assert np.all(model.get(warm.WEIGHT) == 1.0)
        noff = model.ppr_batch(conf, sp2, si2, scores=True)
    finally:
        model.set(warm.PARAMS, params)
    cold = go.ppr_batch(dg, conf, sp2, si2)
    assert trained.converged.all() and noff.converged.all() and cold.converged.all()
    t, o, c = trained.iterations.mean(), noff.iterations.mean(), cold.iterations.mean()
    assert t < o < c, (t, o, c)
    # the same vectors whichever start the iteration took
    a, b = trained.scores.astype(np.float64), noff.scores.astype(np.float64)
    assert np.abs(a - b).sum(axis=1).max() < 2e-6
