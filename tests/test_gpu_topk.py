"""Device top_k / normalize (gops_top_k_*_device, gops_normalize_f64_device)
against a restatement of src/topk.rs:17-61: skip non-finite and non-positive
scores; keep the k largest (at a boundary tie, the entries met first);
ordered by score descending, equal scores by index."""
import numpy as np
import pytest
import torch

import graphops_gb300 as go
from graphops_gb300 import gen
from graphops_gb300.topk import normalize_device, top_k_device, top_k_rows_device

pytestmark = pytest.mark.gpu


def ref_top_k(x, k):
    ok = np.isfinite(x) & (x > 0)
    cand = np.nonzero(ok)[0]
    order = sorted(cand.tolist(), key=lambda i: (-x[i], i))
    return order[:k]


def test_vectors_with_ties_and_invalid_entries():
    rng = np.random.default_rng(0)
    for n, k in [(1, 1), (10, 3), (1000, 100), (100000, 1024), (5000, 7)]:
        x = rng.integers(0, 50, n).astype(np.float64) / 7.0    # many ties
        x[rng.integers(0, n, max(1, n // 20))] = np.nan
        x[rng.integers(0, n, max(1, n // 20))] = -1.0
        x[rng.integers(0, n, max(1, n // 50))] = np.inf
        t = torch.tensor(x, device="cuda")
        got = top_k_device(t.data_ptr(), n, k)
        want = ref_top_k(x, k)
        assert [i for i, _ in got] == want
        assert [v for _, v in got] == [x[i] for i in want]


def test_fewer_valid_than_k_and_degenerate():
    x = np.array([0.0, -2.0, 3.0, np.nan, 1.0])
    t = torch.tensor(x, device="cuda")
    assert top_k_device(t.data_ptr(), 5, 10) == [(2, 3.0), (4, 1.0)]
    assert top_k_device(t.data_ptr(), 5, 0) == []
    z = torch.zeros(4, dtype=torch.float64, device="cuda")
    assert top_k_device(z.data_ptr(), 4, 3) == []


def test_rows_match_host_top100_of_batched_ppr():
    g = gen.rmat(14, 16, seed=9)
    sp, si = gen.seed_sets(g, 48, 1, 16, seed=4)
    dg = go.DeviceGraph.from_csr(g.row_ptr, g.col)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    host = go.ppr_batch(dg, conf, sp, si).scores
    block = torch.tensor(host, device="cuda")
    idx, val, cnt = top_k_rows_device(block.data_ptr(), 48, g.n, 100)
    for r in range(48):
        want = ref_top_k(host[r].astype(np.float64), 100)
        assert cnt[r] == len(want) and idx[r, :cnt[r]].tolist() == want


def test_normalize_device():
    x = np.array([2.0, 3.0, 5.0])                           # the doctest, src/topk.rs:46-52
    t = torch.tensor(x, device="cuda")
    normalize_device(t.data_ptr(), 3)
    y = t.cpu().numpy()
    assert abs(y[0] - 0.2) < 1e-12 and abs(y[2] - 0.5) < 1e-12
    z = torch.tensor([0.0, 0.0], dtype=torch.float64, device="cuda")
    normalize_device(z.data_ptr(), 2)                       # sum 0: unchanged
    assert (z.cpu().numpy() == 0).all()


def test_long_rows_two_stage_ties_across_segments():
    """Rows longer than two 32,768-entry segments run as every segment's top
    k, then the top k of the candidates: the same entries and order as one
    pass, including ties of the k-th value spread over many segments (the
    lowest indices win) and more equal maxima than k."""
    rng = np.random.default_rng(1)
    n = 300000
    x = rng.random(n)
    x[rng.integers(0, n, 5000)] = 2.0            # 5,000 equal maxima over every segment
    x[rng.integers(0, n, 3000)] = np.nan
    got = top_k_device(torch.tensor(x, device="cuda").data_ptr(), n, 1024)
    assert [i for i, _ in got] == ref_top_k(x, 1024)
    y = np.floor(rng.random(n) * 40) / 40.0      # 40 levels: the k-th value tied across segments
    got = top_k_device(torch.tensor(y, device="cuda").data_ptr(), n, 700)
    assert [i for i, _ in got] == ref_top_k(y, 700)
    rows = (np.floor(rng.random((5, 200000)) * 1000) / 1000).astype(np.float32)
    rows[2] = -1.0                               # no valid entry
    rows[3, :150000] = 0.5
    block = torch.tensor(rows, device="cuda")
    idx, val, cnt = top_k_rows_device(block.data_ptr(), 5, 200000, 100)
    for r in range(5):
        want = ref_top_k(rows[r].astype(np.float64), 100)
        assert cnt[r] == len(want) and idx[r, :cnt[r]].tolist() == want
        assert val[r, :cnt[r]].tolist() == [float(rows[r, i]) for i in want]


def test_normalize_long_vector():
    rng = np.random.default_rng(2)
    x = rng.random(3_000_000)
    t = torch.tensor(x, device="cuda")
    normalize_device(t.data_ptr(), x.shape[0])
    y = t.cpu().numpy()
    assert np.abs(y - x / x.sum()).max() <= 1e-15 * np.abs(x / x.sum()).max() * 4
