"""Batched PPR (gops_ppr_batch) against the oracle, set by set.

Every seed set must equal one reference personalized_pagerank_run with
personalization 1 on its seeds (oracle.port.ppr_many): L1 <= 1e-7 per set,
iteration count within +-1 (exact expected), same convergence flag.
"""
import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300 import gen
from oracle import fp64, port

pytestmark = pytest.mark.gpu
L1_TARGET = 1e-7


def check(g, sp, si, tol=1e-7, max_iter=1000, x0=None):
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    conf = go.PageRankConfig(0.85, max_iter, tol)
    r = go.ppr_batch(dg, conf, sp, si, x0=x0)
    ref, its = port.ppr_many(g.row_ptr, g.col, sp, si, 0.85, max_iter, tol, threads=8)
    return r, ref, its


def test_waves_match_reference_per_set():
    g = gen.rmat(12, 16, seed=4)
    sp, si = gen.seed_sets(g, 70, 1, 64, seed=2)          # 3 waves, the last partial
    r, ref, its = check(g, sp, si)
    l1 = np.abs(r.scores.astype(np.float64) - ref).sum(axis=1)
    assert l1.max() <= L1_TARGET, l1.max()
    assert np.array_equal(r.iterations, its.astype(np.int64))
    assert r.converged.all()


def test_edge_cases_empty_repeated_and_capped():
    g = gen.rmat(11, 8, seed=6)
    sets = [[], [5, 5, 7], [0], list(range(40)), [3]]
    sp, si = go.seed_sets_to_csr(sets)
    r, ref, its = check(g, sp, si)
    assert np.abs(r.scores.astype(np.float64) - ref).sum(axis=1).max() <= L1_TARGET
    assert np.array_equal(r.iterations, its.astype(np.int64))
    # empty set = uniform personalization (src/ppr.rs:104-109)
    u, _, _, _ = port.ppr_run(g.row_ptr, g.col, np.zeros(g.n), 0.85, 1000, 1e-7)
    assert np.abs(r.scores[0] - u).sum() <= L1_TARGET
    # max_iterations reached: every set stops at 3, not converged
    r3, ref3, its3 = check(g, sp, si, tol=1e-12, max_iter=3)
    assert (r3.iterations == 3).all() and not r3.converged.any()
    assert np.abs(r3.scores.astype(np.float64) - ref3).sum(axis=1).max() <= L1_TARGET


def test_big_rows_are_chunked():
    n = 20000
    rows = [[0] if u % 3 else [0, (u * 7919) % n] for u in range(n)]
    rows[0] = [1, 2, 3]
    rp = np.zeros(n + 1, np.int64)
    for u, rr in enumerate(rows):
        rp[u + 1] = rp[u] + len(rr)
    col = np.array([v for rr in rows for v in rr], np.int32)
    g = gen.CsrGraph(n, rp, col)
    sets = [[0], [1, 2], [17, 555, 9000], [], [n - 1]]
    sp, si = go.seed_sets_to_csr(sets)
    r, ref, its = check(g, sp, si, tol=1e-9)
    assert np.abs(r.scores.astype(np.float64) - ref).sum(axis=1).max() <= L1_TARGET
    assert np.abs(r.iterations - its.astype(np.int64)).max() <= 1


def test_deterministic():
    g = gen.rmat(12, 16, seed=9)
    sp, si = gen.seed_sets(g, 40, 1, 32, seed=5)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    a = go.ppr_batch(dg, conf, sp, si)
    b = go.ppr_batch(dg, conf, sp, si)
    assert np.array_equal(a.scores, b.scores) and np.array_equal(a.iterations, b.iterations)


def test_warm_start_from_the_fixed_point_stops_early():
    g = gen.rmat(11, 16, seed=3)
    sp, si = gen.seed_sets(g, 8, 1, 16, seed=8)
    x0 = np.zeros((8, g.n), np.float32)
    for i in range(8):
        p = np.zeros(g.n)
        p[si[sp[i]:sp[i + 1]]] = 1.0
        x0[i] = fp64.fixed_point(g.n, g.row_ptr, g.col, 0.85, personalization=p)
    cold, ref, its = check(g, sp, si)
    warm = go.ppr_batch(go.DeviceGraph.from_csr(g.row_ptr, g.col), go.PageRankConfig(0.85, 1000, 1e-7),
                        sp, si, x0=x0)
    assert warm.converged.all()
    assert (warm.iterations < cold.iterations).all()
    # a warm start changes where the iteration stops, not what it converges to
    assert np.abs(warm.scores.astype(np.float64) - x0).sum(axis=1).max() <= 1e-6


def test_warm_starts_over_several_waves():
    """Caller start vectors over 3 waves (the last partial): every wave's
    starts enter through the tiled staging, the host side of the next wave
    is prepared while one runs; each set converges to its own fixed point."""
    g = gen.rmat(11, 16, seed=6)
    ns = 70
    sp, si = gen.seed_sets(g, ns, 1, 16, seed=9)
    x0 = np.zeros((ns, g.n), np.float32)
    fixed = np.zeros((ns, g.n))
    for i in range(ns):
        p = np.zeros(g.n)
        p[si[sp[i]:sp[i + 1]]] = 1.0
        fixed[i] = fp64.fixed_point(g.n, g.row_ptr, g.col, 0.85, personalization=p)
        # half the sets start near their fixed point, half from a flat vector
        x0[i] = fixed[i] if i % 2 == 0 else np.full(g.n, 1.0 / g.n)
    warm = go.ppr_batch(go.DeviceGraph.from_csr(g.row_ptr, g.col), go.PageRankConfig(0.85, 1000, 1e-7),
                        sp, si, x0=x0)
    assert warm.converged.all()
    assert np.abs(warm.scores.astype(np.float64) - fixed).sum(axis=1).max() <= 1e-6
    assert (warm.iterations[0::2] < warm.iterations[1::2].max()).all()


def test_device_pointers_variant():
    torch = pytest.importorskip("torch")
    import ctypes
    from graphops_gb300 import _native
    g = gen.rmat(11, 16, seed=2)
    sp, si = gen.seed_sets(g, 33, 1, 8, seed=1)
    ctx = _native.default_context()
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    host = go.ppr_batch(dg, go.PageRankConfig(0.85, 1000, 1e-7), sp, si)
    out = torch.empty((33, g.n), dtype=torch.float32, device="cuda")
    cfg = _native.Config(0.85, 1000, 1e-7)
    runs = (_native.Run * 33)()
    torch.cuda.synchronize()
    ctx.check(ctx._l.gops_ppr_batch_device(ctx.handle, dg.handle, ctypes.byref(cfg), 33,
                                            _native.ptr(np.ascontiguousarray(sp)),
                                            _native.ptr(np.ascontiguousarray(si)), None,
                                            ctypes.c_void_p(out.data_ptr()), ctypes.cast(runs, ctypes.c_void_p)))
    assert np.array_equal(out.cpu().numpy(), host.scores)


def test_every_tile_gives_the_same_bits():
    """The autotuner may pick any k-tile (32, 64 or 128 sets per wave), chunk
    size of long rows (256 or 1024 edges) and L2 hints on or off.  A row's sum is fixed as
    in-order sums of 256-edge blocks added in order, so every choice gives
    bit-identical scores and step counts, cold and from caller start
    vectors, and every choice matches the oracle set by set."""
    g = gen.rmat(14, 16, seed=12)  # hub rows of several thousand in-edges
    assert np.diff(g.row_ptr).max() > 1024
    sp, si = gen.seed_sets(g, 150, 1, 48, seed=13)  # 2 waves of 128, 5 of 32
    sets = [list(si[sp[q]:sp[q + 1]]) if q % 37 else [] for q in range(150)]  # some empty (uniform)
    sp, si = go.seed_sets_to_csr(sets)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    rng = np.random.default_rng(3)
    x0 = rng.random((150, g.n)).astype(np.float32)
    x0 /= x0.sum(axis=1, keepdims=True)
    ref, its = port.ppr_many(g.row_ptr, g.col, sp, si, 0.85, 1000, 1e-7, threads=8)
    first = None
    tiles = [(c, ch, False) for c in (32, 64, 128) for ch in (256, 1024)] + [(64, 256, True), (128, 1024, True)]
    for cols, chunk, l2 in tiles:
        dg.set_batch_tile(cols, chunk, l2)
        assert dg.batch_tile()[:3] == (cols, chunk, l2)
        r = go.ppr_batch(dg, conf, sp, si)
        w = go.ppr_batch(dg, conf, sp, si, x0=x0)
        assert r.converged.all() and w.converged.all()
        if first is None:
            first = (r, w)
            l1 = np.abs(r.scores.astype(np.float64) - ref).sum(axis=1)
            assert l1.max() <= L1_TARGET, l1.max()
            assert np.array_equal(r.iterations, its.astype(np.int64))
        else:
            assert np.array_equal(r.scores, first[0].scores), (cols, chunk, l2)
            assert np.array_equal(r.iterations, first[0].iterations), (cols, chunk, l2)
            assert np.array_equal(w.scores, first[1].scores), (cols, chunk, l2)
            assert np.array_equal(w.iterations, first[1].iterations), (cols, chunk, l2)
    dg.set_batch_tile(0)  # autotune: the fastest candidate, then L2 hints on it if they pay
    cols, chunk, l2, cost, cost_l2 = dg.batch_tile()
    assert cols in (32, 64, 128) and chunk in (256, 1024)
    assert (cost[0] > 0).all() and cost[{32: 0, 64: 1, 128: 2}[cols], {256: 0, 1024: 1}[chunk]] == cost[cost > 0].min()
    assert cost_l2 > 0 and l2 == (cost_l2 < cost[cost > 0].min())
    r = go.ppr_batch(dg, conf, sp, si)
    assert np.array_equal(r.scores, first[0].scores)


def test_rows_without_in_edges_skipped_bit_for_bit():
    """From step 4 a wave skips the rows without in-edges that seed none of
    its sets (their step residual is exactly 0 from step 2 on); a wave with
    an empty seed set (uniform personalization) skips nothing.  The same 40
    sets -- many seeded on rows without in-edges, some solved from caller
    start vectors -- in one wave alone, and in one wave with an empty set
    added, give the same bits, and match the oracle."""
    g = gen.rmat(14, 8, seed=31)
    n = g.n
    indeg = np.bincount(np.asarray(g.col), minlength=n)
    outdeg = np.diff(np.asarray(g.row_ptr))
    no_in = np.nonzero((indeg == 0) & (outdeg > 0))[0]
    rng = np.random.default_rng(5)
    sets = []
    for i in range(40):
        k = int(rng.integers(1, 9))
        s = list(rng.choice(no_in, size=min(k, len(no_in)), replace=False)) if i % 2 == 0 else []
        s += list(rng.integers(0, n, size=k))
        sets.append([int(v) for v in s])
    sp, si = go.seed_sets_to_csr(sets)
    sp_u, si_u = go.seed_sets_to_csr(sets + [[]])
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    dg.set_batch_tile(64, 256, False)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    a = go.ppr_batch(dg, conf, sp, si)
    b = go.ppr_batch(dg, conf, sp_u, si_u)
    assert np.array_equal(a.scores, b.scores[:40])
    assert np.array_equal(a.iterations, b.iterations[:40]) and a.converged.all()
    # the skipping steps ran (a set seeded only on nodes without edges is its
    # own fixed point and stops after one step)
    assert (a.iterations >= 6).sum() >= 30
    ref, its = port.ppr_many(g.row_ptr, g.col, sp, si, 0.85, 1000, 1e-7, threads=8)
    assert np.abs(a.scores.astype(np.float64) - ref).sum(axis=1).max() <= L1_TARGET
    assert np.array_equal(a.iterations, its.astype(np.int64))
    # caller start vectors (every entry nonzero, rows without in-edges included)
    x0 = np.full((40, n), 1.0 / n, dtype=np.float32)
    x0_u = np.full((41, n), 1.0 / n, dtype=np.float32)
    c = go.ppr_batch(dg, conf, sp, si, x0=x0)
    d = go.ppr_batch(dg, conf, sp_u, si_u, x0=x0_u)
    assert np.array_equal(c.scores, d.scores[:40])
    assert np.array_equal(c.iterations, d.iterations[:40])
    # another start: each result within d/(1-d) tol of the fixed point, like the oracle's
    assert np.abs(c.scores.astype(np.float64) - ref).sum(axis=1).max() <= 1e-6


def test_caller_score_arrays():
    """out = the caller's array: a page-locked one is filled by DMA straight
    from each wave's block (one copy per set, on the copy stream), a pageable
    one through the pinned staging; both hold the bits of a new array, over
    three waves whose sets run in size order."""
    torch = pytest.importorskip("torch")
    g = gen.rmat(12, 16, seed=4)
    sp, si = gen.seed_sets(g, 70, 1, 64, seed=2)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    new = dg.ppr_batch(conf, sp, si)[0]
    pinned = torch.empty((70, g.n), dtype=torch.float32).pin_memory().numpy()
    pinned.fill(np.nan)
    got = dg.ppr_batch(conf, sp, si, out=pinned)[0]
    assert got is pinned and np.array_equal(pinned, new)
    pageable = np.full((70, g.n), np.nan, dtype=np.float32)
    assert np.array_equal(dg.ppr_batch(conf, sp, si, out=pageable)[0], new)
    with pytest.raises(ValueError, match="float32 array of shape"):
        dg.ppr_batch(conf, sp, si, out=np.empty((70, g.n), np.float64))
    with pytest.raises(ValueError, match="float32 array of shape"):
        dg.ppr_batch(conf, sp, si, out=np.empty((69, g.n), np.float32))
