"""Save and load of a trained warm-start model (WarmStart.save / load): the
loaded model has the same parameters, coupling and clusters and predicts the
same start vectors; a checkpoint is refused for another graph.  The file
format itself is tested without a device in test_warm_checkpoint.py."""
import numpy as np
import pytest
import torch

import graphops_gb300 as go
from graphops_gb300 import gen, warm

pytestmark = pytest.mark.gpu


def test_checkpoint_round_trip(tmp_path):
    sb = gen.sbm(3000, 8, 1.2, 16.0, 4.0, seed=5)
    dg = go.DeviceGraph.from_csr(sb.row_ptr, sb.col)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    ws = warm.WarmStart(dg, sb.row_ptr, sb.col, warm.default_config(clusters=16, chunk=64, minibatch=16))
    tsp, tsi = gen.seed_sets(sb, 128, 1, 16, seed=6)
    ws.train(conf, tsp, tsi)
    path = tmp_path / "model.gopswarm"
    ws.save(path)
    ws2 = warm.WarmStart.load(path, dg, sb.row_ptr, sb.col)
    for what in (warm.PARAMS, warm.COUPLING, warm.CLUSTERS):
        assert np.array_equal(ws2.get(what), ws.get(what)), what
    esp, esi = gen.seed_sets(sb, 16, 1, 16, seed=7)
    xa = torch.empty(16 * sb.n, dtype=torch.float32, device="cuda")
    xb = torch.empty_like(xa)
    ra = ws.predict_device(0.85, esp, esi, xa.data_ptr())
    rb = ws2.predict_device(0.85, esp, esi, xb.data_ptr())
    torch.cuda.synchronize()
    assert np.allclose(ra, rb, rtol=1e-12, atol=0.0)
    assert torch.allclose(xa, xb, rtol=1e-6, atol=1e-9)
    other = gen.sbm(3000, 8, 1.2, 16.0, 4.0, seed=6)
    dgo = go.DeviceGraph.from_csr(other.row_ptr, other.col)
    with pytest.raises(ValueError, match="different graph"):
        warm.WarmStart.load(path, dgo, other.row_ptr, other.col)
