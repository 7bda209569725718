"""The warm-start checkpoint file (graphops_gb300.warm.write_checkpoint /
read_checkpoint) and its configuration and graph fingerprints, without a
device.  The save/load round trip of a trained model on the GPU is in
test_gpu_warm_checkpoint.py."""
import struct

import numpy as np
import pytest

from graphops_gb300 import warm


def test_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    arrays = {"params": rng.standard_normal(1000).astype(np.float32),
              "coupling": rng.standard_normal(33).astype(np.float32),
              "clusters": rng.integers(0, 16, 777).astype(np.int32),
              "empty": np.zeros(0, np.float32)}
    meta = {"config": {"clusters": 16}, "n": 777, "m": 5000, "graph_sha256": "ab"}
    p = tmp_path / "m.gopswarm"
    warm.write_checkpoint(p, meta, arrays)
    m2, a2 = warm.read_checkpoint(p)
    assert m2 == meta
    assert set(a2) == set(arrays)
    for k, v in arrays.items():
        assert a2[k].dtype == v.dtype and np.array_equal(a2[k], v)
    assert not (tmp_path / "m.gopswarm.tmp").exists()


def test_rejects_other_files(tmp_path):
    p = tmp_path / "x"
    warm.write_checkpoint(p, {"n": 1}, {"params": np.ones(8, np.float32)})
    data = p.read_bytes()
    bad = tmp_path / "bad"
    bad.write_bytes(b"NOTAWARM" + data[8:])
    with pytest.raises(ValueError, match="not a warm-start checkpoint"):
        warm.read_checkpoint(bad)
    bad.write_bytes(data[:8] + struct.pack("<I", 2) + data[12:])
    with pytest.raises(ValueError, match="version 2 is not supported"):
        warm.read_checkpoint(bad)
    bad.write_bytes(data[:-8])
    with pytest.raises(ValueError, match="truncated"):
        warm.read_checkpoint(bad)
    bad.write_bytes(data[:16] + b"X" + data[17:])  # the JSON header opens with "{"
    with pytest.raises(ValueError, match="corrupt"):
        warm.read_checkpoint(bad)
    with pytest.raises(ValueError, match="1-D float32 or int32"):
        warm.write_checkpoint(bad, {}, {"x": np.ones(3)})


def test_config_round_trip():
    c = warm.default_config(clusters=72, seed=5, lr=0.003, chunk=256)
    d = warm.config_to_dict(c)
    c2 = warm.config_from_dict(d)
    assert warm.config_to_dict(c2) == d and d["clusters"] == 72 and d["seed"] == 5


def test_graph_digest():
    rp = np.array([0, 2, 3, 3], np.int64)
    col = np.array([1, 2, 0], np.int32)
    d = warm.graph_digest(rp, col)
    assert d == warm.graph_digest(rp.astype(np.int32), col.astype(np.int64))  # dtype-independent
    assert d != warm.graph_digest(rp, np.array([1, 2, 1], np.int32))
    assert d != warm.graph_digest(np.array([0, 1, 3, 3], np.int64), col)
