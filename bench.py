"""Benchmark: weighted PageRank on an R-MAT graph, GTEPS on GB300.

Workload (default): R-MAT scale 22 (4,194,304 nodes), edge factor 16,
a/b/c/d = 0.57/0.19/0.19/0.05, self loops and duplicates removed, weights
uniform(0.1, 1.0) in FP32; damping 0.85, tolerance 1e-8 (L1 of the step),
max_iterations 1000.  One step = one full solve to tolerance.
GTEPS = m * iterations / time.

  value     device-resident: the graph is on the device when the timed
            region starts; CUDA events on the library's stream bracket K solves.
  e2e       through the public API from pinned host buffers: every step
            uploads the out-CSR and weights, builds the in-edge CSR on the
            device, solves and copies the scores back.
  roofline  the FP32-phase pull kernel (the dominant one): algorithmic bytes
            per launch 8(N+1) + 8m + 8N over its mean CUDA-event duration,
            against the measured HBM copy bandwidth.
  cpu_baseline  the oracle's C restatement of pagerank_weighted_run (the
            reference is single-threaded) on a bounded number of iterations.
  accuracy  ||F(x) - x||_1 of the FP64 iteration map at the end-to-end result
            x, computed on the host with scipy, and the bound it gives on the
            L1 distance from the exact fixed point; the batched and learned
            sections carry the same check for three of their result columns.

The same line carries dense_small (the n = 2000 dense-matrix case, latency),
ppr_batched (seeds/s on R-MAT 20, with the autotuned tile and the batched
step's roofline), ppr_learned (learned warm start vs plain batched seeds/s on
the block-model graph, with the ablation: the same pipeline with the network
switched off) and stress (R-MAT 25: weighted PageRank with its own roofline,
end-to-end figure, accuracy and CPU sample, then learned vs plain batched PPR
on 256 sets of sizes U[1,128]).  Every accuracy object carries the measured
L1 distance from the oracle's restatement of the reference on the same
inputs, the top-100 order check and the step counts.

--impl reference times that CPU restatement alone, in the same JSON shape.
Multi-GPU: one replica per rank (the solve does not shard without an
exchange); value = all ranks' edges traversed / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "PPR seeds/s to L1 1e-7, learned+batched vs plain, 1 GB300; PageRank GTEPS"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=int, default=22)
    ap.add_argument("--edge-factor", type=int, default=16)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--max-iter", type=int, default=1000)
    ap.add_argument("--seed", type=int, default=22)
    ap.add_argument("--cpu-iters", type=int, default=0,
                    help="iterations of the CPU sample (0: sized to ~10 s)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-PPR measurement")
    ap.add_argument("--batch-scale", type=int, default=20)
    ap.add_argument("--batch-sets", type=int, default=1024)
    ap.add_argument("--no-learned", action="store_true", help="skip the learned warm-start measurement")
    ap.add_argument("--only", choices=["all", "pagerank", "batched", "learned", "stress"], default="all",
                    help="run one section (profiling); the default runs all of them")
    ap.add_argument("--learned-n", type=int, default=500000)
    ap.add_argument("--learned-train", type=int, default=50000)
    ap.add_argument("--learned-sets", type=int, default=4096)
    ap.add_argument("--learned-rmat", type=int, default=0,
                    help="run the learned section on R-MAT of this scale (edge factor 16) instead of the SBM")
    ap.add_argument("--learned-size-hi", type=int, default=32, help="largest seed set of the learned section")
    ap.add_argument("--no-stress", action="store_true", help="skip the R-MAT 25 stress section")
    ap.add_argument("--stress-scale", type=int, default=25)
    ap.add_argument("--stress-train", type=int, default=2048)
    ap.add_argument("--stress-sets", type=int, default=256)
    return ap.parse_args()


def workload_config(a, m):
    return {
        "workload": f"weighted PageRank, R-MAT scale {a.scale} edge factor {a.edge_factor} "
                    f"(0.57/0.19/0.19/0.05, dedup, no self loops), w~U(0.1,1) FP32",
        "nodes": 1 << a.scale, "edges": int(m), "damping": 0.85, "tolerance": a.tol,
        "max_iterations": a.max_iter, "graph_seed": a.seed,
        "l2": "inputs larger than L2 (CSR + weights > 129 MB); no flush",
    }


def dist_init(a):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if a.impl == "gb300" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group(backend)
    return rank, ws


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device, self.rows, self._stop = device, [], threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        # back-to-back queries (each nvidia-smi call takes tens of ms)
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out and not self._stop.is_set():
                    self.rows.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.01)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(self.rows)}


def make_graph(a):
    from graphops_gb300 import gen
    return gen.rmat(a.scale, a.edge_factor, 0.57, 0.19, 0.19, weighted=True, wlo=0.1, whi=1.0,
                    seed=a.seed)


def cpu_sample(g, a, iters):
    """The oracle's pagerank_weighted_run on `iters` iterations, 1 thread."""
    from oracle import port
    w64 = g.weight.astype(np.float64)
    t0 = time.perf_counter()
    _, it, _, _ = port.pagerank_weighted_run(g.row_ptr, g.col, w64, 0.85, iters, a.tol)
    dt = time.perf_counter() - t0
    return g.m * it / dt / 1e9, it, dt


def fp64_residual(row_ptr, col, weights, x, d=0.85, p=None):
    """||F(x) - x||_1 of the reference's iteration map in FP64 on the host
    (scipy), an independent check of a GPU result: F(x) = (1-d) p + d A x +
    d D(x) q with A[v,u] = max(w,0)/ws(u) (weights None: 1/deg(u)), D(x) the
    mass on dangling nodes, p the uniform vector (q = p) or a personalization
    (q = p, src/ppr.rs:125-128).  The error of x against the exact fixed
    point is at most this residual / (1 - d)."""
    import scipy.sparse as sps
    n = row_ptr.shape[0] - 1
    src = np.repeat(np.arange(n), np.diff(row_ptr))
    w = np.ones(col.shape[0]) if weights is None else np.maximum(np.asarray(weights, np.float64), 0.0)
    ws = np.bincount(src, weights=w, minlength=n)
    safe = np.where(ws > 0, ws, 1.0)
    M = sps.csr_matrix((w / safe[src], col, row_ptr), shape=(n, n))  # M[u, v] = A[v, u]
    x = np.asarray(x, np.float64)
    q = np.full(n, 1.0 / n) if p is None else np.asarray(p, np.float64) / np.sum(p)
    fx = (1.0 - d) * q + d * (M.T @ x) + d * x[ws == 0].sum() * q
    return float(np.abs(fx - x).sum())


def top_order_matches(a, b, k=100, tie=0.0):
    """The k largest entries of a in the order of b's, ties in b within
    1e-15 relative counting as equal (top_k sorts unstably, src/topk.rs:40),
    or within `tie` (absolute: for FP32 results, twice their largest error)."""
    ia = np.argsort(-a, kind="stable")[:k]
    ib = np.argsort(-b, kind="stable")[:k]
    return bool(all(x == y or abs(b[x] - b[y]) <= max(1e-15 * max(abs(b[x]), 1e-300), tie)
                    for x, y in zip(ia, ib)))


def columns_accuracy(g, sp, si, scores, cols, d=0.85, iterations=None):
    """Checks of a few result columns of a batched solve (seed set c: p = 1
    per occurrence of each seed, normalised, src/ppr.rs:48-65): the FP64
    residual ||F(x) - x||_1 and its bound on the distance from the exact
    vector, and the measured L1 distance from the oracle's C restatement of
    personalized_pagerank_run on the same sets (with top-100 order and, when
    `iterations` is given, the step counts)."""
    from oracle import port
    t0 = time.perf_counter()
    worst = 0.0
    for c in cols:
        p = np.zeros(g.n)
        np.add.at(p, si[sp[c]:sp[c + 1]], 1.0)
        worst = max(worst, fp64_residual(g.row_ptr, g.col, None, scores[c], d=d, p=p))
    cols = [int(c) for c in cols]
    sp2 = np.zeros(len(cols) + 1, np.int64)
    sp2[1:] = np.cumsum([sp[c + 1] - sp[c] for c in cols])
    si2 = np.concatenate([si[sp[c]:sp[c + 1]] for c in cols]).astype(np.int32)
    ref, its = port.ppr_many(g.row_ptr, g.col, sp2, si2, d, 1000, 1e-7, threads=len(cols))
    l1 = [float(np.abs(scores[c].astype(np.float64) - ref[q]).sum()) for q, c in enumerate(cols)]
    out = {"columns": cols, "worst_fp64_residual_l1": worst, "l1_vs_fixed_point_bound": worst / (1.0 - d),
           "l1_vs_restatement": l1, "l1_vs_restatement_max": max(l1),
           "top100_match": all(top_order_matches(scores[c].astype(np.float64), ref[q],
                                                 tie=2.0 * float(np.abs(scores[c] - ref[q]).max()))
                               for q, c in enumerate(cols)),
           "top100_ties": "FP32 scores: entries may swap only where the restatement's scores differ by less than "
                          "twice the column's largest error",
           "restatement_iterations": [int(x) for x in its]}
    if iterations is not None:
        out["iterations"] = [int(iterations[c]) for c in cols]
    out["check_s"] = round(time.perf_counter() - t0, 2)
    return out


def cpu_all_cores(g, a):
    """A clearly separate all-cores CPU figure: the same iteration in pull
    form over an in-edge CSR (built first, not timed), rows split over every
    host thread, run to convergence.  Not the reference's code path (which is
    single-threaded); reported beside it."""
    from oracle import port
    threads = max(1, os.cpu_count() or 1)
    _, it, _, _, secs = port.pagerank_weighted_run_mt(g.row_ptr, g.col, g.weight.astype(np.float64), 0.85,
                                                      a.max_iter, a.tol, threads)
    return {"value": round(g.m * it / secs / 1e9, 6), "unit": "GTEPS", "cores": threads, "kind": "port",
            "sample": f"{it} iterations (a full solve, {secs:.2f} s), pull form of pagerank_weighted_run over "
                      f"an in-edge CSR, rows split over {threads} threads, FP64"}


def cpu_iters_for(g, a):
    if a.cpu_iters:
        return a.cpu_iters
    # roughly 10 s of single-thread work at ~100 M edge updates/s
    return int(max(1, min(20, 1.0e9 / max(g.m, 1))))


def batch_workload(a):
    return {"workload": f"batched personalized PageRank, R-MAT scale {a.batch_scale} edge factor 16 "
                        f"(0.57/0.19/0.19/0.05, dedup, no self loops), unweighted; {a.batch_sets} seed sets "
                        f"of sizes U[1,64], nodes drawn proportional to out-degree",
            "nodes": 1 << a.batch_scale, "damping": 0.85, "tolerance_per_set": 1e-7,
            "max_iterations": 1000, "graph_seed": 20, "seed_set_seed": "7 + 1000 * rank"}


def shard_seed(base, rank):
    """Seed of a rank's own seed sets: the sets are the units the batched paths
    shard (graph replicated, no data-path collective), so every rank solves
    distinct sets of the same distribution (weak scaling)."""
    return base + 1000 * rank


def batch_inputs(a, rank=0):
    from graphops_gb300 import gen
    g = gen.rmat(a.batch_scale, 16, seed=20)
    sp, si = gen.seed_sets(g, a.batch_sets, 1, 64, seed=shard_seed(7, rank))
    return g, sp, si


def batch_cpu(g, sp, si, nsets, threads):
    """The oracle's personalized_pagerank_run, one call per seed set, spread
    over host threads (independent calls; each call is single-threaded)."""
    from oracle import port
    t0 = time.perf_counter()
    _, its = port.ppr_many(g.row_ptr, g.col, sp[:nsets + 1], si[:sp[nsets]], 0.85, 1000, 1e-7,
                           threads=threads, want_scores=False)
    dt = time.perf_counter() - t0
    return nsets / dt, dt


def run_dense_small(a, ctx, rank):
    """Plain PageRank on the reference's CPU-sized case: directed Erdos-Renyi
    n=2000, p=0.005, 1% of nodes forced dangling, given as a dense
    AdjacencyMatrix (d=0.85, tol 1e-6, max_iterations 100).  Too small for a
    roofline: latency per solve, device-resident (graph on the device) and
    end to end through the public API (dense matrix upload, device
    compaction to CSR, solve, scores back), beside the C restatement of
    pagerank_run with its O(N^2) neighbour scan on one host thread."""
    import torch
    import graphops_gb300 as go
    from graphops_gb300 import _native, gen
    g = gen.erdos_renyi(2000, 0.005, 0.01, seed=0)
    M = gen.dense_adjacency(g)
    conf = go.PageRankConfig(0.85, 100, 1e-6)
    dg = _native.DeviceGraph.from_dense(M, ctx=ctx)
    for _ in range(5):
        dg.pagerank_run(conf, out=False)
    reps = 50
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        _, it, _, _ = dg.pagerank_run(conf, out=True)
    dev_ms = (time.perf_counter() - t0) * 1e3 / reps
    am = go.AdjacencyMatrix(M)
    for _ in range(3):
        go.pagerank_run(am, conf)
    t0 = time.perf_counter()
    for _ in range(reps):
        r = go.pagerank_run(am, conf)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / reps
    out = {"workload": "plain PageRank, directed Erdos-Renyi n=2000 p=0.005, 1% forced dangling, dense "
                       "AdjacencyMatrix, d=0.85, tol 1e-6, max_iterations 100, seed 0",
           "edges": int(g.m), "iterations": int(r.iterations),
           "ms_per_solve_device_resident": round(dev_ms, 4), "ms_per_solve_e2e": round(e2e_ms, 4),
           "e2e_h2d_bytes": int(M.nbytes), "e2e_d2h_bytes": 8 * 2000}
    if rank == 0 and not a.no_cpu:
        from oracle import port  # the C restatement (CPU baseline only)
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < 2.0:
            port.pagerank_run_dense(M, 0.85, 100, 1e-6)
            k += 1
        out["cpu_baseline"] = {"ms_per_solve": round((time.perf_counter() - t0) * 1e3 / k, 3), "cores": 1,
                               "kind": "port", "sample": f"{k} solves of pagerank_run on the dense matrix, "
                                                         f"C restatement incl. the O(N^2) neighbour scan"}
    return out


def batch_roofline(g, st, kt):
    """The batched step's roofline by the per-step formula 8(N+1) + 4m +
    8*N*k (row offsets, column indices, the k-tile's block read and written;
    k = the wave's columns) over the mean CUDA-event duration of the
    FP32-phase launches (every column of a wave counted active: an upper
    bound on the bytes)."""
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    n, m = g.n, g.m
    b = 8 * (n + 1) + 4 * m + 8 * n * kt
    ms = st.f32_ms / max(1, st.f32_launches)
    ach = b / (ms * 1e-3) / 1e9 if st.f32_launches else None
    # the formula reads the block once; the step gathers one k-tile row per
    # in-edge (m rows of 4k bytes): with those counted as well, the rate
    # against the same peak shows how far the gathers are from the copy rate
    gb = b + 4 * m * kt
    achg = gb / (ms * 1e-3) / 1e9 if st.f32_launches else None
    return {"bound": "hbm", "kernel": f"spmm_f32 ({kt} columns per wave)",
            "bytes_per_launch": int(b), "mean_launch_ms": round(ms, 5),
            "achieved": round(ach, 1) if ach else None, "peak": peak,
            "unit": "GB/s", "frac": round(ach / peak, 4) if ach else None,
            "with_gathered_rows": {"bytes_per_launch": int(gb), "achieved": round(achg, 1) if achg else None,
                                   "frac": round(achg / peak, 4) if achg else None,
                                   "note": "8(N+1) + 4m + 8Nk + 4mk: every in-edge gathers its source's k-tile row"},
            "df_phase_mean_ms": round(st.df_ms / max(1, st.df_launches), 5), "df_launches": int(st.df_launches),
            "note": "the formula counts every row; from step 4 the step skips the rows without in-edges "
                    "that seed none of the wave's sets (their entries are exact zeros already), so it "
                    "moves fewer bytes than the formula names",
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s"}


def tile_info(dg):
    """The batched path's autotuned tile: sets per wave (k-tile), the chunk
    size of long rows, and the tuner's measured cost of every candidate."""
    kt, chunk, l2, cost, cost_l2 = dg.batch_tile()
    names = [f"cols{32 << i}_chunk{c}" for i in range(3) for c in (256, 1024)]
    tuned = {nm: round(float(v) * 1e3, 3) for nm, v in zip(names, cost.ravel()) if v > 0}
    if cost_l2 > 0:
        tuned[f"cols{kt}_chunk{chunk}_l2hints"] = round(cost_l2 * 1e3, 3)
    return kt, {"cols": kt, "chunk": chunk, "l2_hints": l2, "tuner_us_per_set_step": tuned}


def pinned_copy(x):
    """A page-locked copy of a host array (a NumPy view of pinned memory)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()


def pinned_empty(shape):
    """A page-locked float32 host array."""
    import torch
    return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()


def run_batch(a, ctx, rank, ws):
    """Batched PPR seeds/s: device-resident graph; end to end with the score
    blocks copied back; CPU reference on a sample of the same seed sets."""
    import graphops_gb300 as go
    from graphops_gb300 import _native
    g, sp, si = batch_inputs(a, rank)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col, ctx=ctx)
    wu = min(128, a.batch_sets)
    dg.ppr_batch(conf, sp[:wu + 1], si[:sp[wu]], out=False)  # autotuned tile, plan, workspace, captured chunks
    kt, tile = tile_info(dg)
    # seeds/s from a run with captured chunks; the per-launch CUDA-event
    # timing of the roofline from a second run with direct launches
    _, its, _, conv = dg.ppr_batch(conf, sp, si, out=False)
    st = ctx.stats()
    ctx.set_timing(True)
    dg.ppr_batch(conf, sp, si, out=False)
    st_t = ctx.stats()
    ctx.set_timing(False)
    t = max_over_ranks(st.solve_ms, ws)
    # end to end: the graph uploaded from page-locked host arrays and the
    # scores of every set written into a page-locked array, both allocated
    # once before the timed call (as a serving loop reuses its buffers)
    rp_h, col_h = pinned_copy(g.row_ptr), pinned_copy(g.col)
    s_h = pinned_empty((a.batch_sets, g.n))
    t0 = time.perf_counter()
    dg2 = _native.DeviceGraph.from_csr(rp_h, col_h, ctx=ctx)
    s, _, _, _ = dg2.ppr_batch(conf, sp, si, out=s_h)
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    acc = (columns_accuracy(g, sp, si, s, (0, a.batch_sets // 2, a.batch_sets - 1), iterations=its)
           if rank == 0 else None)
    out = {"config": batch_workload(a), "seeds_per_s": round(ws * a.batch_sets / (t * 1e-3), 2),
           "ms": round(t, 3), "iterations_mean": float(its.mean()), "iterations_max": int(its.max()),
           "all_converged": bool(conv.all()), "kernel_launches": int(st.kernel_launches),
           "spmm_fp32_launch_ms": round(st_t.f32_ms / max(1, st_t.f32_launches), 4), "tile": tile,
           "roofline": batch_roofline(g, st_t, kt), "accuracy": acc,
           "e2e": {"seeds_per_s": round(ws * a.batch_sets / e2e_s, 2),
                   "h2d_bytes_per_step": int(g.row_ptr.nbytes + g.col.nbytes + sp.nbytes + si.nbytes),
                   "d2h_bytes_per_step": int(s.nbytes),
                   "includes": "graph upload from page-locked arrays and device CSR build, seed sets up, every "
                               "score block into a page-locked host array (buffers allocated before the call)"}}
    del s
    if rank == 0 and not a.no_cpu:
        threads = max(1, os.cpu_count() or 1)
        ns = min(a.batch_sets, 2 * threads)
        v, dt = batch_cpu(g, sp, si, ns, threads)
        out["cpu_baseline"] = {"value": round(v, 3), "unit": "seeds/s", "cores": threads, "kind": "port",
                               "sample": f"{ns} seed sets, one personalized_pagerank_run each "
                                         f"(C restatement, FP64), {threads} threads, {dt:.1f} s"}
        v1, dt1 = batch_cpu(g, sp, si, 2, 1)
        out["cpu_baseline"]["one_core"] = {"value": round(v1, 3), "unit": "seeds/s", "cores": 1,
                                           "sample": f"2 seed sets on one thread, {dt1:.1f} s"}
    return out


def learned_workload(a):
    graph = (f"R-MAT scale {a.learned_rmat} edge factor 16 (0.57/0.19/0.19/0.05, dedup, no self loops)"
             if a.learned_rmat else
             f"stochastic block model n={a.learned_n}, 64 blocks with Zipf(1.2) sizes, intra-block mean "
             f"out-degree 16, inter-block 4 (directed)")
    hi = a.learned_size_hi
    return {"workload": f"learned warm-start batched personalized PageRank, {graph}, unit weights; trained on "
                        f"{a.learned_train} PPR vectors of seed sets of sizes U[1,{hi}] solved by the batched "
                        f"GPU path; evaluated on {a.learned_sets} held-out sets of sizes U[1,{hi}]; nodes "
                        f"drawn proportional to out-degree",
            "nodes": (1 << a.learned_rmat) if a.learned_rmat else a.learned_n, "damping": 0.85,
            "tolerance_per_set": 1e-7, "max_iterations": 1000,
            "graph_seed": 3, "train_seed": 31, "eval_seed": "77 + 1000 * rank",
            "model": "2-layer MPNN (hidden 128, BF16 operands, FP32 accumulation) per-node weight, "
                     "72 k-means clusters (best of 8 seeded runs) of a 16-wide random-projection code, least-squares "
                     "cluster coupling, exact 3-hop push"}


def run_learned(a, ctx, rank, ws):
    """Learned warm start vs plain batched PPR on the same graph and seed
    sets: seeds/s of each (device-resident graph, scores left on the device;
    the learned figure includes the warm-start inference), iterations, and
    an end-to-end figure with the score blocks copied to the host."""
    import graphops_gb300 as go
    from graphops_gb300 import _native, gen, warm
    g = gen.rmat(a.learned_rmat, 16, seed=25) if a.learned_rmat else gen.sbm(a.learned_n, 64, 1.2, 16.0, 4.0, seed=3)
    conf = go.PageRankConfig(0.85, 1000, 1e-7)
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col, ctx=ctx)
    t0 = time.perf_counter()
    # the push scratch and the targets hold chunk x n x 12 bytes: keep them to ~8 GB
    chunk = int(max(32, min(512, 8e9 / (12.0 * g.n))))
    # 72 clusters: the best of 64-256 in a sweep on this graph (validation sets
    # drawn like the evaluation sets); the library default is 128
    model = warm.WarmStart(dg, g.row_ptr, g.col, warm.default_config(chunk=chunk, clusters=72))
    create_s = time.perf_counter() - t0
    sp_t, si_t = gen.seed_sets(g, a.learned_train, 1, a.learned_size_hi, seed=31)
    t0 = time.perf_counter()
    tst = model.train(conf, sp_t, si_t)
    train_s = time.perf_counter() - t0
    sp, si = gen.seed_sets(g, a.learned_sets, 1, a.learned_size_hi, seed=shard_seed(77, rank))
    # warm-up of both paths (plans, workspaces)
    dg.ppr_batch(conf, sp[:65], si[:sp[64]], out=False)
    model.ppr_batch(conf, sp[:65], si[:sp[64]], scores=False)
    _, its_p, _, conv_p = dg.ppr_batch(conf, sp, si, out=False)
    st_p = ctx.stats()
    _, tile = tile_info(dg)
    lr = model.ppr_batch(conf, sp, si, scores=False)
    st_l = ctx.stats()
    tp = max_over_ranks(st_p.solve_ms, ws)
    tl = max_over_ranks(st_l.solve_ms, ws)
    # end to end: both through the public API, every score block into a
    # page-locked host array allocated once before the timed calls
    s_h = pinned_empty((len(sp) - 1, g.n))
    t0 = time.perf_counter()
    s = model.ppr_batch(conf, sp, si, scores=s_h).scores
    e2e_l = max_over_ranks(time.perf_counter() - t0, ws)
    d2h = int(s.nbytes)
    acc = (columns_accuracy(g, sp, si, s, (0, a.learned_sets // 2, a.learned_sets - 1), iterations=lr.iterations)
           if rank == 0 else None)
    del s
    t0 = time.perf_counter()
    s, _, _, _ = dg.ppr_batch(conf, sp, si, out=s_h)
    e2e_p = max_over_ranks(time.perf_counter() - t0, ws)
    del s
    # what the trained network gains: the same pipeline with the network off
    # (w = 1 for every node: w3 = b3 = 0; same push, clusters and coupling)
    params = model.get(warm.PARAMS)
    off = params.copy()
    off[warm.P_W3:warm.P_B3 + 1] = 0.0
    model.set(warm.PARAMS, off)
    model.ppr_batch(conf, sp[:65], si[:sp[64]], scores=False)  # refreshes w for the new parameters
    lo = model.ppr_batch(conf, sp, si, scores=False)
    st_o = ctx.stats()
    model.set(warm.PARAMS, params)
    to = max_over_ranks(st_o.solve_ms, ws)
    n_sets = a.learned_sets
    out = {"config": learned_workload(a),
           "learned_seeds_per_s": round(ws * n_sets / (tl * 1e-3), 2),
           "plain_seeds_per_s": round(ws * n_sets / (tp * 1e-3), 2),
           "ratio": round(tp / tl, 4),
           "learned_ms": round(tl, 3), "plain_ms": round(tp, 3),
           "iterations_mean_learned": float(lr.iterations.mean()),
           "iterations_mean_plain": float(its_p.mean()),
           "rejected": int(lr.rejected.sum()), "accuracy_learned": acc, "tile": tile,
           "ablation": {"trained_iterations_mean": float(lr.iterations.mean()),
                        "network_off_iterations_mean": float(lo.iterations.mean()),
                        "cold_iterations_mean": float(its_p.mean()),
                        "trained_seeds_per_s": round(ws * n_sets / (tl * 1e-3), 2),
                        "network_off_seeds_per_s": round(ws * n_sets / (to * 1e-3), 2),
                        "cold_seeds_per_s": round(ws * n_sets / (tp * 1e-3), 2),
                        "network_off_rejected": int(lo.rejected.sum()),
                        "how": "network off = every node's weight w = 1 (w3 = b3 = 0): the same exact push, "
                               "clusters and least-squares coupling, each cluster's tail mass spread evenly"},
           "all_converged": bool(lr.converged.all() and conv_p.all()),
           "kernel_launches_learned": int(st_l.kernel_launches),
           "train": {"sets": int(tst.sets), "adam_steps": int(tst.steps),
                     "loss_first": round(tst.loss_first, 6), "loss_last": round(tst.loss_last, 6),
                     "targets_ms": round(tst.target_ms, 1), "fit_ms": round(tst.fit_ms, 1),
                     "wall_s": round(train_s, 2), "model_build_s": round(create_s, 2)},
           "e2e": {"learned_seeds_per_s": round(ws * n_sets / e2e_l, 2),
                   "plain_seeds_per_s": round(ws * n_sets / e2e_p, 2),
                   "h2d_bytes_per_step": int(sp.nbytes + si.nbytes), "d2h_bytes_per_step": d2h,
                   "includes": "seed sets up, inference, every score block into a page-locked host array "
                               "(allocated before the calls); the graph and the trained model stay on the "
                               "device (built once, before the timed calls)"}}
    if rank == 0 and not a.no_cpu:
        threads = max(1, os.cpu_count() or 1)
        ns = min(n_sets, threads)
        v, dt = batch_cpu(g, sp, si, ns, threads)
        out["cpu_baseline"] = {"value": round(v, 3), "unit": "seeds/s", "cores": threads, "kind": "port",
                               "sample": f"{ns} seed sets, one personalized_pagerank_run each "
                                         f"(C restatement, FP64), {threads} threads, {dt:.1f} s"}
        v1, dt1 = batch_cpu(g, sp, si, 2, 1)
        out["cpu_baseline"]["one_core"] = {"value": round(v1, 3), "unit": "seeds/s", "cores": 1,
                                           "sample": f"2 seed sets on one thread, {dt1:.1f} s"}
    return out


def peak_hbm():
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(peaks["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs"
    except Exception:
        return 6800.0, "fallback 6800 GB/s"


def run_stress(a, ctx, rank, ws):
    """The large-scale stress configuration: R-MAT scale 25 (33,554,432
    nodes, edge factor 16, 0.57/0.19/0.19/0.05, dedup, no self loops,
    w~U(0.1,1) FP32).  Weighted PageRank at tol 1e-8: GTEPS device-resident
    and end to end (upload of the out-CSR and weights, device build, solve,
    scores back), the FP32 step's roofline, the accuracy against the oracle's
    all-cores pull form of pagerank_weighted_run, and a bounded one-thread
    CPU sample of the serial restatement.  Then learned vs plain batched PPR
    (the reference's PPR is unweighted: the same graph's structure) on 256
    seed sets of sizes U[1,128], the model trained on 2,048 sets."""
    import ctypes
    import torch
    import graphops_gb300 as go
    from graphops_gb300 import _native, gen, warm
    t0 = time.perf_counter()
    g = gen.rmat(a.stress_scale, 16, 0.57, 0.19, 0.19, weighted=True, wlo=0.1, whi=1.0, seed=25)
    gen_s = time.perf_counter() - t0
    n, m = g.n, g.m
    w64 = g.weight.astype(np.float64)
    conf = go.PageRankConfig(0.85, a.max_iter, 1e-8)
    out = {"config": {"workload": f"R-MAT scale {a.stress_scale} edge factor 16 (0.57/0.19/0.19/0.05, dedup, no "
                                  f"self loops), w~U(0.1,1) FP32: weighted PageRank tol 1e-8, then learned vs plain "
                                  f"batched PPR on {a.stress_sets} seed sets of sizes U[1,128]",
                      "nodes": n, "edges": int(m), "damping": 0.85, "graph_seed": 25, "generate_s": round(gen_s, 1)}}
    # ---- weighted PageRank, device-resident
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col, w64, ctx=ctx)
    dg.pagerank_weighted_run(conf, out=False)
    ctx.set_timing(True)
    steps, iters, solve_ms, f32_ms, f32_n, df_ms, df_n = 3, 0, 0.0, 0.0, 0, 0.0, 0
    for _ in range(steps):
        _, it, _, conv = dg.pagerank_weighted_run(conf, out=False)
        st = ctx.stats()
        iters += it
        solve_ms += st.solve_ms
        f32_ms += st.f32_ms
        f32_n += st.f32_launches
        df_ms += st.df_ms
        df_n += st.df_launches
    ctx.set_timing(False)
    t = max_over_ranks(solve_ms, ws)
    peak, peak_src = peak_hbm()
    b = 8 * (n + 1) + 8 * m + 8 * n
    mean_f32 = f32_ms / max(1, f32_n)
    ach = b / (mean_f32 * 1e-3) / 1e9
    pr = {"gteps": round(ws * m * iters / (t * 1e-3) / 1e9, 3), "ms_per_solve": round(t / steps, 3),
          "iterations": int(iters // steps), "converged": bool(conv),
          "roofline": {"bound": "hbm", "kernel": "iterate_kernel<PrecF32, weighted>", "bytes_per_launch": int(b),
                       "mean_launch_ms": round(mean_f32, 5), "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                       "frac": round(ach / peak, 4), "peak_source": peak_src,
                       "df_phase_mean_ms": round(df_ms / max(1, df_n), 5), "df_launches": int(df_n)}}
    # ---- end to end through the public API from pinned host buffers
    rp_h = torch.from_numpy(g.row_ptr).pin_memory()
    col_h = torch.from_numpy(g.col).pin_memory()
    w_h = torch.from_numpy(w64).pin_memory()
    out_h = torch.empty(n, dtype=torch.float64).pin_memory()
    lib = ctx._l
    cfg_c = _native.Config(conf.damping, conf.max_iterations, conf.tolerance)

    def e2e_step():
        h = ctypes.c_void_p()
        ctx.check(lib.gops_graph_upload(ctx.handle, n, ctypes.c_void_p(rp_h.data_ptr()),
                                        ctypes.c_void_p(col_h.data_ptr()), ctypes.c_void_p(w_h.data_ptr()),
                                        ctypes.byref(h)))
        up = ctx.stats()
        r = _native.Run()
        ctx.check(lib.gops_pagerank_weighted_run(ctx.handle, h, ctypes.byref(cfg_c),
                                                 ctypes.c_void_p(out_h.data_ptr()), ctypes.byref(r)))
        st = ctx.stats()
        lib.gops_graph_destroy(h)
        return int(r.iterations), up.h2d_bytes + st.h2d_bytes, st.d2h_bytes

    e2e_step()
    barrier(ws)
    t0 = time.perf_counter()
    e_it, h2d, d2h = 0, 0, 0
    for _ in range(2):
        it, hb, db = e2e_step()
        e_it += it
        h2d += hb
        d2h += db
    e_s = max_over_ranks(time.perf_counter() - t0, ws)
    pr["e2e"] = {"value": round(ws * m * e_it / e_s / 1e9, 3), "unit": "GTEPS", "h2d_bytes_per_step": int(h2d // 2),
                 "d2h_bytes_per_step": int(d2h // 2),
                 "includes": "upload of the out-CSR and FP64 weights, device CSR build, solve, scores to the host"}
    del rp_h, col_h, w_h
    if rank == 0 and not a.no_cpu:
        from oracle import port
        threads = max(1, os.cpu_count() or 1)
        t0 = time.perf_counter()
        ref, rit, _, rconv, secs = port.pagerank_weighted_run_mt(g.row_ptr, g.col, w64, 0.85, a.max_iter, 1e-8,
                                                                 threads)
        x = out_h.numpy()
        pr["accuracy"] = {"l1_vs_restatement": float(np.abs(x - ref).sum()), "top100_match": top_order_matches(x, ref),
                          "iterations": int(e_it // 2), "restatement_iterations": int(rit),
                          "sum": float(x.sum()), "min": float(x.min()),
                          "reference": "the oracle's all-cores pull form of pagerank_weighted_run (FP64; equal to the "
                                       "serial restatement within 1e-12 in L1 with the same step count)",
                          "check_s": round(time.perf_counter() - t0, 1)}
        pr["cpu_baseline_all_cores"] = {"value": round(m * rit / secs / 1e9, 4), "unit": "GTEPS", "cores": threads,
                                        "kind": "port", "sample": f"a full solve ({rit} iterations, {secs:.1f} s), "
                                                                  f"pull form over an in-edge CSR, {threads} threads"}
        del ref
        t0 = time.perf_counter()
        _, cit, _, _ = port.pagerank_weighted_run(g.row_ptr, g.col, w64, 0.85, 3, 1e-8)
        dt = time.perf_counter() - t0
        pr["cpu_baseline"] = {"value": round(m * cit / dt / 1e9, 4), "unit": "GTEPS", "cores": 1, "kind": "port",
                              "sample": f"{cit} iterations of pagerank_weighted_run ({dt:.1f} s, including its "
                                        f"weight-sum pass), C restatement, FP64, single thread"}
    out["pagerank"] = pr
    del w64
    # ---- learned vs plain batched PPR on the same graph (structure only)
    pconf = go.PageRankConfig(0.85, 1000, 1e-7)
    t0 = time.perf_counter()
    chunk = int(max(32, min(512, 8e9 / (12.0 * n))))
    model = warm.WarmStart(dg, g.row_ptr, g.col, warm.default_config(chunk=chunk, clusters=72))
    create_s = time.perf_counter() - t0
    sp_t, si_t = gen.seed_sets(g, a.stress_train, 1, 128, seed=31)
    t0 = time.perf_counter()
    tst = model.train(pconf, sp_t, si_t)
    train_s = time.perf_counter() - t0
    sp, si = gen.seed_sets(g, a.stress_sets, 1, 128, seed=shard_seed(77, rank))
    dg.ppr_batch(pconf, sp[:33], si[:sp[32]], out=False)
    model.ppr_batch(pconf, sp[:33], si[:sp[32]], scores=False)
    _, its_p, _, conv_p = dg.ppr_batch(pconf, sp, si, out=False)
    st_p = ctx.stats()
    lr = model.ppr_batch(pconf, sp, si, scores=False)
    st_l = ctx.stats()
    _, tile = tile_info(dg)
    tp, tl = max_over_ranks(st_p.solve_ms, ws), max_over_ranks(st_l.solve_ms, ws)
    ns = a.stress_sets
    bat = {"plain_seeds_per_s": round(ws * ns / (tp * 1e-3), 2), "learned_seeds_per_s": round(ws * ns / (tl * 1e-3), 2),
           "ratio": round(tp / tl, 4), "iterations_mean_plain": float(its_p.mean()),
           "iterations_mean_learned": float(lr.iterations.mean()), "rejected": int(lr.rejected.sum()),
           "all_converged": bool(conv_p.all() and lr.converged.all()), "tile": tile,
           "train": {"sets": int(tst.sets), "wall_s": round(train_s, 2), "model_build_s": round(create_s, 2),
                     "loss_first": round(tst.loss_first, 6), "loss_last": round(tst.loss_last, 6)}}
    model.close()
    if rank == 0 and not a.no_cpu:
        from oracle import port
        threads = max(1, os.cpu_count() or 1)
        k = min(ns, threads)
        t0 = time.perf_counter()
        port.ppr_many(g.row_ptr, g.col, sp[:k + 1], si[:sp[k]], 0.85, 2, 1e-7, threads=threads, want_scores=False)
        dt = time.perf_counter() - t0
        per_set = dt / 2.0 * float(its_p.mean())
        bat["cpu_baseline"] = {"value": round(k / per_set, 4), "unit": "seeds/s", "cores": threads, "kind": "port",
                               "sample": f"{k} seed sets on {threads} threads, 2 iterations of "
                                         f"personalized_pagerank_run each ({dt:.1f} s), scaled to the plain GPU "
                                         f"path's mean of {its_p.mean():.1f} iterations per set"}
    out["ppr"] = bat
    dg.close()
    return out


def run_reference(a):
    rank, ws = dist_init(a)
    if rank != 0:
        return
    g = make_graph(a)
    iters = cpu_iters_for(g, a)
    for _ in range(max(0, a.warmup)):
        cpu_sample(g, a, 1)
    vals, its, secs = [], 0, 0.0
    for _ in range(max(1, a.steps)):
        v, it, dt = cpu_sample(g, a, iters)
        vals.append(v)
        its += it
        secs += dt
    value = g.m * its / secs / 1e9
    line = {
        "metric": METRIC, "impl": "reference", "value": round(value, 6), "unit": "GTEPS",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": round(secs / max(1, a.steps) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(a, g.m),
        "cpu_baseline": {"value": round(value, 6), "unit": "GTEPS", "cores": 1, "kind": "port",
                         "sample": f"{iters} iterations of pagerank_weighted_run per step "
                                   f"(C restatement, FP64, single thread: the reference path is "
                                   f"single-threaded)"},
        "e2e": {"value": round(value, 6), "unit": "GTEPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    line["cpu_baseline"]["all_cores"] = cpu_all_cores(g, a)
    print(json.dumps(line))


def run_section(a):
    """--only batched|learned|stress: one section's object alone (for profiling)."""
    rank, ws = dist_init(a)
    import torch
    from graphops_gb300 import _native
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    ctx = _native.Context(dev)
    fn = {"batched": run_batch, "learned": run_learned, "stress": run_stress}[a.only]
    out = fn(a, ctx, rank, ws)
    if rank == 0:
        print(json.dumps({"metric": METRIC, "section": a.only, "n_gpus": ws, a.only: out}))


def run_gpu(a):
    if a.only in ("batched", "learned", "stress"):
        return run_section(a)
    if a.only == "pagerank":
        a.no_batch = a.no_learned = a.no_stress = True
    rank, ws = dist_init(a)
    import ctypes
    import torch
    import graphops_gb300 as go
    from graphops_gb300 import _native

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    ctx = _native.Context(dev)
    g = make_graph(a)
    n, m = g.n, g.m
    conf = go.PageRankConfig(0.85, a.max_iter, a.tol)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", dev))

    # ---- device-resident solves ----
    dg = _native.DeviceGraph.from_csr(g.row_ptr, g.col, g.weight.astype(np.float64), ctx=ctx)
    for _ in range(max(3, a.warmup)):
        dg.pagerank_weighted_run(conf, out=False)
    ctx.set_timing(True)
    barrier(ws)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters, launches, f32_ms, f32_n, df_ms, df_n = 0, 0, 0.0, 0, 0.0, 0
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        for _ in range(a.steps):
            _, it, diff, conv = dg.pagerank_weighted_run(conf, out=False)
            st = ctx.stats()
            iters += it
            launches += st.kernel_launches
            f32_ms += st.f32_ms
            f32_n += st.f32_launches
            df_ms += st.df_ms
            df_n += st.df_launches
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize()
    barrier(ws)
    ctx.set_timing(False)
    t_ms = max_over_ranks(ev0.elapsed_time(ev1), ws)
    value = ws * m * iters / (t_ms * 1e-3) / 1e9
    ms_per_step = t_ms / a.steps

    # ---- roofline of the FP32-phase pull kernel ----
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    bytes_per_launch = 8 * (n + 1) + 8 * m + 8 * n
    mean_f32 = f32_ms / max(1, f32_n)
    achieved = bytes_per_launch / (mean_f32 * 1e-3) / 1e9 if f32_n else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(f"rmat{a.scale}_weighted_f32")
        except Exception:
            traffic = None

    # ---- end to end through the public API from pinned host buffers ----
    rp_h = torch.from_numpy(g.row_ptr).pin_memory()
    col_h = torch.from_numpy(g.col).pin_memory()
    w_h = torch.from_numpy(g.weight.astype(np.float64)).pin_memory()
    out_h = torch.empty(n, dtype=torch.float64).pin_memory()
    lib = ctx._l
    cfg_c = _native.Config(conf.damping, conf.max_iterations, conf.tolerance)

    def e2e_step():
        h = ctypes.c_void_p()
        ctx.check(lib.gops_graph_upload(ctx.handle, n, ctypes.c_void_p(rp_h.data_ptr()),
                                        ctypes.c_void_p(col_h.data_ptr()),
                                        ctypes.c_void_p(w_h.data_ptr()), ctypes.byref(h)))
        up = ctx.stats()
        r = _native.Run()
        ctx.check(lib.gops_pagerank_weighted_run(ctx.handle, h, ctypes.byref(cfg_c),
                                                 ctypes.c_void_p(out_h.data_ptr()), ctypes.byref(r)))
        st = ctx.stats()
        lib.gops_graph_destroy(h)
        return int(r.iterations), up.h2d_bytes + st.h2d_bytes, st.d2h_bytes, up.kernel_launches + st.kernel_launches

    e2e_steps = max(1, min(a.steps, 3))
    for _ in range(2):
        e2e_step()
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_iters, h2d, d2h = 0, 0, 0
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(e2e_steps):
        it, hb, db, _ = e2e_step()
        e_iters += it
        h2d += hb
        d2h += db
    e1.record(stream)
    e1.synchronize()
    wall = time.perf_counter() - t0
    e_ms = max_over_ranks(max(e0.elapsed_time(e1), wall * 1e3), ws)
    e2e_value = ws * m * e_iters / (e_ms * 1e-3) / 1e9

    # ---- accuracy of the timed end-to-end result, checked on the host ----
    quality = None
    if rank == 0:
        t0 = time.perf_counter()
        res = fp64_residual(g.row_ptr, g.col, g.weight, out_h.numpy(), d=conf.damping)
        quality = {"fp64_residual_l1": res, "l1_vs_fixed_point_bound": res / (1.0 - conf.damping),
                   "sum": float(out_h.numpy().sum()), "min": float(out_h.numpy().min()),
                   "iterations": int(e_iters // e2e_steps),
                   "check_s": round(time.perf_counter() - t0, 2),
                   "how": "||F(x) - x||_1 of the FP64 iteration map (scipy) at the e2e result x; "
                          "||x - x*||_1 <= residual / (1 - d); l1_vs_restatement against the oracle's "
                          "C restatement of pagerank_weighted_run on the same graph"}

    # ---- CPU baseline (rank 0): one full solve of the C restatement on one
    # thread; its result is also the parity reference of the accuracy object
    cpu = None
    if rank == 0 and not a.no_cpu:
        from oracle import port
        t0 = time.perf_counter()
        ref, rit, _, _ = port.pagerank_weighted_run(g.row_ptr, g.col, g.weight.astype(np.float64), conf.damping,
                                                    a.max_iter, a.tol)
        dt = time.perf_counter() - t0
        cpu = {"value": round(m * rit / dt / 1e9, 6), "unit": "GTEPS", "cores": 1, "kind": "port",
               "sample": f"a full solve ({rit} iterations, {dt:.1f} s) of pagerank_weighted_run, C restatement, "
                         f"FP64, single thread (the reference path is single-threaded)"}
        cpu["all_cores"] = cpu_all_cores(g, a)
        quality["l1_vs_restatement"] = float(np.abs(out_h.numpy() - ref).sum())
        quality["top100_match"] = top_order_matches(out_h.numpy(), ref)
        quality["restatement_iterations"] = int(rit)
        del ref

    dense_small = run_dense_small(a, ctx, rank)
    batch = None
    if not a.no_batch:
        batch = run_batch(a, ctx, rank, ws)
    learned = None
    if not a.no_learned:
        learned = run_learned(a, ctx, rank, ws)
    stress = None
    if not a.no_stress:
        del dg
        stress = run_stress(a, ctx, rank, ws)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": "GTEPS", "n_gpus": ws,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(ms_per_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (double-float first phase, exact 64-bit fixed-point sums)",
            "data": "synthetic", "config": workload_config(a, m),
            "iterations_per_solve": iters / a.steps,
            "e2e": {"value": round(e2e_value, 4), "unit": "GTEPS",
                    "h2d_bytes_per_step": int(h2d / e2e_steps), "d2h_bytes_per_step": int(d2h / e2e_steps)},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None,
                         "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4) if achieved else None,
                         "traffic": traffic, "kernel": "iterate_kernel<PrecF32, weighted>",
                         "bytes_per_launch": bytes_per_launch,
                         "mean_launch_ms": round(mean_f32, 5), "launches": f32_n,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800 GB/s",
                         "df_phase_mean_ms": round(df_ms / max(1, df_n), 5), "df_launches": df_n},
            "gpu_launches": launches,
            "accuracy": quality,
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
            "dense_small": dense_small,
            "ppr_batched": batch,
            "ppr_learned": learned,
            "stress": stress,
        }
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)
