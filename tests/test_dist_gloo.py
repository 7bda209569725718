"""The multi-rank host path of bench.py on CPU: two gloo ranks (the GPU run
uses NCCL with one rank per GPU; every box here has one GPU).  The paths
shard by seed set with no data-path collective, so what runs across ranks
is the timing protocol: barrier, max over ranks, rank 0 printing one line,
and distinct seed sets per rank."""
import json
import os
import socket
import subprocess
import sys
from types import SimpleNamespace

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    sys.path.insert(0, ROOT)
    import bench
    r, ws = bench.dist_init(SimpleNamespace(impl="reference"))
    bench.barrier(ws)
    mx = bench.max_over_ranks(1.5 + r, ws)
    results[r] = (r, ws, mx, bench.shard_seed(7, r))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_timing_protocol():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = free_port()
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_worker, args=(port, results), nprocs=2, join=True)
        got = dict(results)
    assert got[0][:3] == (0, 2, 2.5) and got[1][:3] == (1, 2, 2.5)
    assert got[0][3] != got[1][3]


def test_reference_arm_two_ranks_prints_once():
    pytest.importorskip("torch")
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--scale", "10", "--steps", "1", "--warmup", "3",
           "--cpu-iters", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["value"] > 0
    line = lines[0]
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["n_gpus"] == 2 and line["steps"] == 1 and line["warmup"] == 3
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["all_cores"]["value"] > 0


class _FakeCtx:
    """Stands in for the device context: a rank's solve takes 10 + 5 * rank ms."""

    def __init__(self, rank):
        self.rank = rank

    def stats(self):
        return SimpleNamespace(solve_ms=10.0 + 5.0 * self.rank, kernel_launches=7, f32_ms=1.0, f32_launches=2,
                               df_ms=0.5, df_launches=1)

    def set_timing(self, on):
        pass


class _FakeDeviceGraph:
    """Stands in for a device graph: records the seed sets it was asked to
    solve and returns zero scores (the sharding, not the solve, is tested)."""
    seen = []

    def __init__(self, n):
        self.n = n

    @classmethod
    def from_csr(cls, row_ptr, col, w=None, ctx=None):
        return cls(len(row_ptr) - 1)

    def ppr_batch(self, conf, sp, si, out=True):
        import numpy as np
        ns = len(sp) - 1
        _FakeDeviceGraph.seen.append(tuple(int(x) for x in si[:64]))
        if isinstance(out, np.ndarray):  # the caller's array
            out[:] = 0.0
            s = out
        else:
            s = np.zeros((ns, self.n), np.float32) if out else None
        return s, np.full(ns, 11, np.int64), np.zeros(ns), np.ones(ns, bool)

    def batch_tile(self):
        import numpy as np
        return 128, 256, False, np.zeros((3, 2), np.float32), 0.0


def _batch_worker(rank, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    sys.path.insert(0, ROOT)
    import bench
    from graphops_gb300 import _native
    _native.DeviceGraph = _FakeDeviceGraph
    # page-locked host buffers need a GPU: plain arrays stand in for them
    import numpy as np
    bench.pinned_copy = np.ascontiguousarray
    bench.pinned_empty = lambda shape: np.empty(shape, np.float32)
    r, ws = bench.dist_init(SimpleNamespace(impl="reference"))
    a = SimpleNamespace(impl="gb300", batch_scale=10, batch_sets=64, no_cpu=True)
    out = bench.run_batch(a, _FakeCtx(r), r, ws)
    results[r] = (out["seeds_per_s"], out["ms"], _FakeDeviceGraph.seen[-1], out["accuracy"] is not None)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_batched_section_shards_seed_sets_over_two_ranks():
    """bench.run_batch on two gloo ranks with the device solve stubbed out:
    each rank solves its own seed sets (no data-path collective), the time is
    the slowest rank's, seeds/s counts every rank's sets, and only rank 0
    checks accuracy against the oracle."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = free_port()
    with mp.Manager() as m:
        results = m.dict()
        mp.spawn(_batch_worker, args=(port, results), nprocs=2, join=True)
        got = dict(results)
    want = round(2 * 64 / 0.015, 2)  # both ranks' sets over the slower rank's 15 ms
    assert got[0][0] == want and got[1][0] == want
    assert got[0][1] == 15.0 and got[1][1] == 15.0
    assert got[0][2] != got[1][2]
    assert got[0][3] and not got[1][3]
