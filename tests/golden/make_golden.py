"""Generates tests/golden/golden.json.

The reference crate holds no numeric golden vectors (its tests check
invariants only) and cannot be built here (Rust, no toolchain), so the
fixtures come from two sources that do not share code with the C oracle:

* the pure-Python restatement oracle/pyref.py, run on the graphs of the
  reference's own tests, doctests and example (and a few small random graphs
  in the style of its proptests) -- scores stored bit-exactly as float.hex;
* exact rational fixed points (fractions.Fraction Gaussian elimination) of the
  same Markov chains, for the closed-form pins (e.g. a 3-cycle is 1/3 each).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import random
import sys
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyref  # noqa: E402


def exact_fixed_point(neighbors, weights, damping, personalization=None):
    """Exact solution of x = F(x) over the rationals (damping as a Fraction)."""
    n = len(neighbors)
    d = Fraction(damping)
    if weights is None:
        out = [Fraction(len(nb)) for nb in neighbors]
        P = [[Fraction(0)] * n for _ in range(n)]
        for u, nb in enumerate(neighbors):
            for v in nb:
                P[u][v] += Fraction(1) / out[u]
        dang = [len(nb) == 0 for nb in neighbors]
    else:
        ws = []
        for u in range(n):
            ws.append(sum((Fraction(max(w, 0.0)) for w in weights[u]), Fraction(0)))
        P = [[Fraction(0)] * n for _ in range(n)]
        for u, nb in enumerate(neighbors):
            for v, w in zip(nb, weights[u]):
                w = Fraction(max(w, 0.0))
                if ws[u] > 0 and w > 0:
                    P[u][v] += w / ws[u]
        dang = [ws[u] == 0 for u in range(n)]
    if personalization is None:
        red = [Fraction(1, n)] * n
    else:
        ps = [Fraction(x) for x in personalization]
        s = sum(ps)
        red = [x / s for x in ps] if s > 0 else [Fraction(1, n)] * n
    # (I - d P^T - d red dang^T) x = (1-d) red
    A = [[Fraction(int(i == j)) - d * P[j][i] - (d * red[i] if dang[j] else 0) for j in range(n)]
         for i in range(n)]
    b = [(1 - d) * red[i] for i in range(n)]
    for c in range(n):
        piv = next(r for r in range(c, n) if A[r][c] != 0)
        A[c], A[piv] = A[piv], A[c]
        b[c], b[piv] = b[piv], b[c]
        for r in range(n):
            if r != c and A[r][c] != 0:
                f = A[r][c] / A[c][c]
                A[r] = [a - f * ac for a, ac in zip(A[r], A[c])]
                b[r] -= f * b[c]
    return [b[i] / A[i][i] for i in range(n)]


def dense_nb(M):
    return pyref.dense_neighbors(M)


def dense_w(M):
    return [[M[u][v] for v in nb] for u, nb in enumerate(dense_nb(M))]


def case(name, source, neighbors, weights=None, personalization=None, damping=0.85,
         max_iterations=100, tolerance=1e-6, exact=False):
    if personalization is not None:
        r = pyref.personalized_pagerank_run(neighbors, personalization, damping, max_iterations, tolerance)
        kind = "ppr"
    elif weights is not None:
        r = pyref.pagerank_weighted_run(neighbors, weights, damping, max_iterations, tolerance)
        kind = "weighted"
    else:
        r = pyref.pagerank_run(neighbors, damping, max_iterations, tolerance)
        kind = "plain"
    c = {
        "name": name, "source": source, "kind": kind, "neighbors": neighbors, "weights": weights,
        "personalization": personalization, "damping": damping, "max_iterations": max_iterations,
        "tolerance": tolerance, "scores_hex": [float(x).hex() for x in r.scores],
        "iterations": r.iterations, "diff_l1_hex": float(r.diff_l1).hex(), "converged": r.converged,
    }
    if exact:
        fp = exact_fixed_point(neighbors, weights, damping, personalization)
        c["fixed_point"] = [f"{x.numerator}/{x.denominator}" for x in fp]
    return c


def random_proptest_graph(rng, n):
    """Like the reference's proptest (src/pagerank.rs:381-389): up to 40
    random (u, v) pairs in 0..10, kept when u, v < n and u != v, 0/1 matrix."""
    M = [[0.0] * n for _ in range(n)]
    for _ in range(rng.randrange(0, 40)):
        u, v = rng.randrange(10), rng.randrange(10)
        if u < n and v < n and u != v:
            M[u][v] = 1.0
    return M


def build_cases():
    cases = []
    cyc = [[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]]
    cases.append(case("doctest_3cycle", "src/pagerank.rs:103-112", dense_nb(cyc), exact=True))
    wadj = [[0.0, 2.0, 1.0], [0.0, 0.0, 1.0], [0.0, 0.0, 0.0]]
    cases.append(case("weighted_sums_to_one", "src/pagerank.rs:344-359", dense_nb(wadj), dense_w(wadj), exact=True))
    hadj = [[0.0, 2.0, 1.0], [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]
    cases.append(case("weight_biases_heavier", "src/pagerank.rs:361-377", dense_nb(hadj), dense_w(hadj), exact=True))
    cases.append(case("ppr_doctest_3cycle", "src/ppr.rs:53-64", dense_nb(cyc), personalization=[1.0, 0.0, 0.0], exact=True))
    ex = [[0.0, 1.0, 1.0, 0.0], [0.0, 0.0, 1.0, 0.0], [1.0, 0.0, 0.0, 0.0], [0.0, 0.0, 1.0, 0.0]]
    cases.append(case("example_4node", "examples/pagerank.rs:14-26", dense_nb(ex), tolerance=1e-8, exact=True))
    chain = [[1], [2], []]
    cases.append(case("petgraph_chain_pr", "tests/invariants.rs:20-32", chain, exact=True))
    cases.append(case("petgraph_chain_ppr", "tests/invariants.rs:35-50", chain, personalization=[1.0, 0.0, 0.0], exact=True))
    rng = random.Random(1234)
    for i in range(12):
        n = rng.randrange(1, 10)
        M = random_proptest_graph(rng, n)
        cases.append(case(f"proptest_like_{i}", "src/pagerank.rs:379-395", dense_nb(M), exact=(n <= 6)))
    # multigraph adapter order, duplicates, a self loop, dangling nodes
    multi = [[1, 1, 2, 0], [2], [], [0, 2, 2], [4]]
    cases.append(case("multigraph_plain", "src/graph.rs:26-39 (duplicates counted)", multi))
    mw = [[0.5, 0.5, 2.0, 1.0], [1.0], [], [-1.0, 0.0, 3.0], [0.0]]
    cases.append(case("multigraph_weighted_clamps", "src/pagerank.rs:227-261 (max(w,0), w>0)", multi, mw))
    cases.append(case("multigraph_ppr", "src/ppr.rs:90-156", multi, personalization=[0.0, 2.0, 0.0, 1.0, 0.0]))
    cases.append(case("ppr_zero_sum_uniform", "src/ppr.rs:104-109", multi, personalization=[0.0] * 5))
    cases.append(case("nonconverged_max_iter_3", "src/pagerank.rs:142-186", multi, max_iterations=3, tolerance=1e-12))
    cases.append(case("damping_zero", "src/pagerank.rs:150-152", multi, damping=0.0))
    cases.append(case("damping_one", "src/pagerank.rs:150-152", [[1], [2], [0]], damping=1.0))
    cases.append(case("single_node", "src/pagerank.rs:132-133", [[]]))
    cases.append(case("all_dangling", "src/pagerank.rs:144-152", [[], [], [], []]))
    rng = random.Random(99)
    nb = [[rng.randrange(40) for _ in range(rng.randrange(0, 6))] for _ in range(40)]
    cases.append(case("random40_plain", "src/pagerank.rs:122-187", nb, tolerance=1e-10, max_iterations=200))
    ws = [[rng.choice([0.1, 0.5, 1.0, 2.5, 0.0]) for _ in row] for row in nb]
    cases.append(case("random40_weighted", "src/pagerank.rs:210-289", nb, ws, tolerance=1e-10, max_iterations=200))
    pers = [float(rng.randrange(0, 3)) for _ in range(40)]
    cases.append(case("random40_ppr", "src/ppr.rs:90-156", nb, personalization=pers, tolerance=1e-10, max_iterations=200))
    return cases


def main():
    cases = build_cases()
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, f, indent=1)
    print(f"wrote {len(cases)} cases")


if __name__ == "__main__":
    main()
