"""The oracle is pinned before anything is checked against it.

* against the golden fixtures (pure-Python restatement, bit for bit, and the
  exact rational fixed points of the reference's own test graphs);
* against the reference's known-answer tests and invariants
  (src/pagerank.rs:98-113,344-395, src/ppr.rs:48-65,163-181,
  tests/invariants.rs:20-50, examples/pagerank.rs);
* against the independent FP64 fixed-point oracle on generated graphs.
"""
import math
import random
from fractions import Fraction

import numpy as np
import pytest

from conftest import case_csr, load_golden
from oracle import fp64, port, pyref

GOLDEN = load_golden()


def run_case(c):
    rp, col, w = case_csr(c)
    kw = dict(damping=c["damping"], max_iterations=c["max_iterations"], tolerance=c["tolerance"])
    if c["kind"] == "ppr":
        return port.ppr_run(rp, col, c["personalization"], **kw)
    if c["kind"] == "weighted":
        return port.pagerank_weighted_run(rp, col, w, **kw)
    return port.pagerank_run(rp, col, **kw)


@pytest.mark.parametrize("c", GOLDEN, ids=[c["name"] for c in GOLDEN])
def test_c_port_matches_golden_bitwise(c):
    s, it, diff, conv = run_case(c)
    assert [float(x).hex() for x in s] == c["scores_hex"]
    assert it == c["iterations"]
    assert float(diff).hex() == c["diff_l1_hex"]
    assert conv == c["converged"]


@pytest.mark.parametrize("c", [c for c in GOLDEN if "fixed_point" in c], ids=lambda c: c["name"])
def test_golden_near_exact_fixed_point(c):
    s = [float.fromhex(x) for x in c["scores_hex"]]
    exact = [float(Fraction(q)) for q in c["fixed_point"]]
    diff = float.fromhex(c["diff_l1_hex"])
    d = c["damping"]
    # a contraction with factor <= d: ||x_k - x*|| <= d/(1-d) * ||x_k - x_{k-1}||
    bound = (d / (1 - d)) * diff + 1e-13 if d < 1 else 1e-9
    assert sum(abs(a - b) for a, b in zip(s, exact)) <= bound


def test_known_answers_of_the_reference():
    g = {c["name"]: c for c in GOLDEN}
    s = [float.fromhex(x) for x in g["doctest_3cycle"]["scores_hex"]]
    assert abs(sum(s) - 1.0) < 1e-6 and all(abs(x - 1 / 3) < 1e-15 for x in s)
    s = [float.fromhex(x) for x in g["weighted_sums_to_one"]["scores_hex"]]
    assert abs(sum(s) - 1.0) < 1e-6
    s = [float.fromhex(x) for x in g["weight_biases_heavier"]["scores_hex"]]
    assert s[1] >= s[2]
    s = [float.fromhex(x) for x in g["ppr_doctest_3cycle"]["scores_hex"]]
    assert s[0] > s[1]
    s = [float.fromhex(x) for x in g["example_4node"]["scores_hex"]]
    assert int(np.argmax(s)) == 2
    for name in ("petgraph_chain_pr", "petgraph_chain_ppr"):
        s = [float.fromhex(x) for x in g[name]["scores_hex"]]
        assert all(math.isfinite(x) and x >= 0 for x in s) and abs(sum(s) - 1) <= 1e-6


def test_proptest_invariant_random_small_graphs():
    """src/pagerank.rs:379-395 on 300 random 0/1 matrices."""
    rng = random.Random(7)
    for _ in range(300):
        n = rng.randrange(1, 10)
        M = np.zeros((n, n))
        for _ in range(rng.randrange(0, 40)):
            u, v = rng.randrange(10), rng.randrange(10)
            if u < n and v < n and u != v:
                M[u, v] = 1.0
        s, it, diff, conv = port.pagerank_run_dense(M)
        assert s.shape == (n,)
        assert abs(s.sum() - 1.0) < 1e-6
        assert (s >= -1e-12).all()


def test_c_port_equals_pure_python_on_random_multigraphs():
    rng = random.Random(3)
    for trial in range(40):
        n = rng.randrange(1, 30)
        nb = [[rng.randrange(n) for _ in range(rng.randrange(0, 5))] for _ in range(n)]
        ws = [[rng.choice([0.0, 0.25, 1.0, 3.0, -1.0]) for _ in row] for row in nb]
        pers = [float(rng.randrange(0, 3)) for _ in range(n)]
        rp = np.zeros(n + 1, dtype=np.int64)
        for i, row in enumerate(nb):
            rp[i + 1] = rp[i] + len(row)
        col = np.array([v for row in nb for v in row], dtype=np.int32)
        w = np.array([x for row in ws for x in row])
        a = port.pagerank_run(rp, col, tolerance=1e-9)
        b = pyref.pagerank_run(nb, 0.85, 100, 1e-9)
        assert list(a[0]) == b.scores and a[1] == b.iterations
        a = port.pagerank_weighted_run(rp, col, w, tolerance=1e-9)
        b = pyref.pagerank_weighted_run(nb, ws, 0.85, 100, 1e-9)
        assert list(a[0]) == b.scores and a[1] == b.iterations
        a = port.ppr_run(rp, col, pers, tolerance=1e-9)
        b = pyref.personalized_pagerank_run(nb, pers, 0.85, 100, 1e-9)
        assert list(a[0]) == b.scores and a[1] == b.iterations


def test_nan_weight_is_clamped_like_rust_max():
    # f64::max(NaN, 0.0) == 0.0: a NaN weight drops the edge
    rp = np.array([0, 2, 3, 3]); col = np.array([1, 2, 2], dtype=np.int32)
    a = port.pagerank_weighted_run(rp, col, [float("nan"), 1.0, 1.0])
    b = port.pagerank_weighted_run(rp, col, [0.0, 1.0, 1.0])
    assert np.array_equal(a[0], b[0])


def test_dense_adapter_semantics():
    M = np.array([[0.0, 2.0, -1.0, np.nan], [0.0, 0.0, 0.0, 1e-300], [1.0, 1.0, 1.0, 0.0], [0, 0, 0, 0]])
    rp, col, w = port.dense_to_csr(M)
    assert rp.tolist() == [0, 1, 2, 5, 5]
    assert col.tolist() == [1, 3, 0, 1, 2]
    assert w.tolist() == [2.0, 1e-300, 1.0, 1.0, 1.0]
    assert pyref.dense_neighbors(M.tolist()) == [[1], [3], [0, 1, 2], []]


def test_oracle_against_fp64_fixed_point_on_generated_graph():
    from graphops_gb300 import gen
    g = gen.rmat(12, 16, weighted=True, seed=5)
    s, it, diff, conv = port.pagerank_weighted_run(g.row_ptr, g.col, g.weight.astype(np.float64),
                                                   tolerance=1e-12, max_iterations=500)
    x = fp64.fixed_point(g.n, g.row_ptr, g.col, 0.85, weights=g.weight)
    assert conv and np.abs(s - x).sum() < 1e-10
    p = np.zeros(g.n); p[[3, 17, 99]] = 1.0
    s, it, diff, conv = port.ppr_run(g.row_ptr, g.col, p, tolerance=1e-12, max_iterations=500)
    x = fp64.fixed_point(g.n, g.row_ptr, g.col, 0.85, personalization=p)
    assert conv and np.abs(s - x).sum() < 1e-10


def test_ppr_many_threads_equal_single():
    from graphops_gb300 import gen
    g = gen.rmat(10, 8, seed=2)
    sp, si = gen.seed_sets(g, 12, 1, 8, seed=4)
    a, ia = port.ppr_many(g.row_ptr, g.col, sp, si, tolerance=1e-8, threads=1)
    b, ib = port.ppr_many(g.row_ptr, g.col, sp, si, tolerance=1e-8, threads=4)
    assert np.array_equal(a, b) and np.array_equal(ia, ib)
    p = np.zeros(g.n); p[si[sp[3]:sp[4]]] = 1.0
    s, it, _, _ = port.ppr_run(g.row_ptr, g.col, p, tolerance=1e-8)
    assert np.array_equal(a[3], s) and ia[3] == it


def test_all_cores_timing_form_matches_serial_restatement():
    """The pull-form, multi-threaded figure bench.py reports beside the
    single-threaded restatement runs the same iteration (other summation
    order): same step count, L1 within rounding."""
    from graphops_gb300 import gen
    g = gen.rmat(12, 16, weighted=True, seed=12)
    w = g.weight.astype(np.float64)
    a = port.pagerank_weighted_run(g.row_ptr, g.col, w, 0.85, 1000, 1e-8)
    for t in (1, 3, 8):
        b = port.pagerank_weighted_run_mt(g.row_ptr, g.col, w, 0.85, 1000, 1e-8, threads=t)
        assert b[1] == a[1] and b[3] == a[3]
        assert np.abs(b[0] - a[0]).sum() <= 1e-12


def test_bench_accuracy_check_bounds_the_error():
    """bench.py's host check of the timed result (||F(x) - x||_1 of the FP64
    iteration map, scipy) is ~0 at the FP64 fixed point, and residual/(1-d)
    bounds the L1 distance of a converged restatement iterate from it, for
    weighted PageRank and for a personalization."""
    import bench
    from graphops_gb300 import gen
    g = gen.rmat(10, 8, weighted=True, seed=3)
    w = g.weight.astype(np.float64)
    x = fp64.fixed_point(g.n, g.row_ptr, g.col, 0.85, weights=w)
    assert bench.fp64_residual(g.row_ptr, g.col, w, x) < 1e-13
    xr = port.pagerank_weighted_run(g.row_ptr, g.col, w, 0.85, 1000, 1e-8)[0]
    res = bench.fp64_residual(g.row_ptr, g.col, w, xr)
    assert 0.0 < res < 1e-8 and np.abs(xr - x).sum() <= res / 0.15
    p = np.zeros(g.n); p[[3, 5]] = 1.0
    xp = fp64.fixed_point(g.n, g.row_ptr, g.col, 0.85, personalization=p)
    assert bench.fp64_residual(g.row_ptr, g.col, None, xp, p=p) < 1e-13
    # a wrong vector is caught
    assert bench.fp64_residual(g.row_ptr, g.col, w, np.full(g.n, 1.0 / g.n)) > 1e-3


def test_bench_column_accuracy_of_seed_sets():
    """The batched sections' check: seed set c means p = 1 per occurrence of
    each seed (a repeated node counts twice); converged restatement columns
    pass with residual below the tolerance, and swapped columns are caught."""
    import bench
    from graphops_gb300 import gen
    g = gen.rmat(10, 8, seed=4)
    sp = np.array([0, 2, 5, 6], np.int64)
    si = np.array([3, 9, 7, 7, 100, 42], np.int32)
    x, _ = port.ppr_many(g.row_ptr, g.col, sp, si, 0.85, 1000, 1e-9)
    acc = bench.columns_accuracy(g, sp, si, x, (0, 1, 2))
    assert acc["worst_fp64_residual_l1"] < 1e-9
    bad = bench.columns_accuracy(g, sp, si, x[::-1].copy(), (0, 1, 2))
    assert bad["worst_fp64_residual_l1"] > 1e-2


def test_golden_fixture_is_what_its_generator_makes():
    """tests/golden/golden.json is exactly the output of
    tests/golden/make_golden.py (pure-Python restatement + exact rationals),
    so the fixture's provenance is checked on every run."""
    import importlib.util
    import json
    import os
    from conftest import ROOT
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    made = json.loads(json.dumps({"generator": "tests/golden/make_golden.py", "cases": mg.build_cases()}))
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        assert json.load(f) == made
