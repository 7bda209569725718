"""Katz and eigenvector centrality: the oracle (C restatement) against the
reference's own tests and doctests (src/katz.rs:213-330,
src/eigenvector.rs:128-215) and closed forms; the Python validation messages."""
import math

import numpy as np
import pytest

import graphops_gb300 as go
from oracle import port


def csr(adj):
    rp = np.zeros(len(adj) + 1, dtype=np.int64)
    for i, r in enumerate(adj):
        rp[i + 1] = rp[i] + len(r)
    col = np.array([v for r in adj for v in r], dtype=np.int32)
    return rp, col


def test_katz_path_center_outscores_endpoints():  # src/katz.rs:233-253 and the doctest
    s, it, diff, conv = port.katz_run(*csr([[1], [0, 2], [1, 3], [2]]))
    assert len(s) == 4 and (s >= 0).all()
    assert s[1] > s[0] and s[2] > s[3]


def test_katz_triangle_all_equal_closed_form():  # src/katz.rs:257-270
    s, it, diff, conv = port.katz_run(*csr([[1, 2], [0, 2], [0, 1]]))
    assert conv
    assert np.abs(s - s[0]).max() < 1e-6
    # fixed point beta / (1 - 2 alpha) = 1.25; the returned iterate is within tol of it
    assert abs(s[0] - 1.25) < 1e-6


def test_katz_checked_rejects_alpha_at_least_one():  # src/katz.rs:274-292
    for a in (1.0, 2.5):
        with pytest.raises(go.InvalidParameter):
            go.KatzConfig(alpha=a).validate()


def test_katz_random_graphs_finite_nonnegative():  # the proptest, src/katz.rs:294-322
    rng = np.random.default_rng(0)
    for _ in range(200):
        n = int(rng.integers(1, 10))
        adj = [set() for _ in range(n)]
        for _ in range(int(rng.integers(0, 30))):
            u, v = int(rng.integers(0, 10)), int(rng.integers(0, 10))
            if u < n and v < n and u != v:
                adj[u].add(v)
                adj[v].add(u)
        s, *_ = port.katz_run(*csr([sorted(a) for a in adj]))
        assert len(s) == n and np.isfinite(s).all() and (s >= 0).all()


def test_katz_no_steps_and_empty():
    s, it, diff, conv = port.katz_run(*csr([[1], [0]]), max_iterations=0)
    assert it == 0 and math.isinf(diff) and not conv and (s == 1.0).all()
    s, it, diff, conv = port.katz_run(np.zeros(1, np.int64), np.zeros(0, np.int32))
    assert len(s) == 0 and it == 0 and conv


def test_eigenvector_triangle_and_doctest():  # src/eigenvector.rs:33-47, 145-156
    s, it, diff, conv = port.eigenvector_run(*csr([[1, 2], [0, 2], [0, 1]]), 100, 1e-8)
    assert conv
    assert np.abs(s - 1 / math.sqrt(3)).max() < 1e-6


def test_eigenvector_star_and_l2():  # src/eigenvector.rs:158-166, 204-213
    s, *_ = port.eigenvector_run(*csr([[1, 2, 3, 4], [0], [0], [0], [0]]))
    assert s[0] > s[1] and abs(s[1] - s[2]) < 1e-6
    s, *_ = port.eigenvector_run(*csr([[1, 2, 3], [0, 2], [0, 1, 3], [0, 2]]))
    assert abs(np.sqrt((s * s).sum()) - 1.0) < 1e-6


def test_eigenvector_isolated_and_empty():  # src/eigenvector.rs:168-202
    s, it, diff, conv = port.eigenvector_run(*csr([[], [], []]))
    assert np.all((np.abs(s) < 1e-10) | (np.abs(s - 1 / math.sqrt(3)) < 1e-10))
    assert conv and it == 1
    s, it, diff, conv = port.eigenvector_run(np.zeros(1, np.int64), np.zeros(0, np.int32))
    assert len(s) == 0 and conv and it == 0


def test_hits_star_and_empty():  # src/centrality.rs:245-275
    hub, auth, it, d, conv = port.hits_run(*csr([[1, 2, 3, 4], [], [], [], []]), 100, 1e-10)
    assert len(hub) == 5
    assert all(hub[0] > hub[i] for i in range(1, 5))
    assert all(auth[i] > auth[0] for i in range(1, 5))
    hub, auth, it, d, conv = port.hits_run(np.zeros(1, np.int64), np.zeros(0, np.int32), 100, 1e-10)
    assert len(hub) == 0 and len(auth) == 0
