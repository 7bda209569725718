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
