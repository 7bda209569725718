"""Learned warm start for batched personalized PageRank (gops_warm_* in
include/gops.h).

No counterpart in the reference crate: it produces the start vectors that
``ppr_batch`` accepts as ``x0``.  For a seed set with normalised indicator s,

    x0 = (1-d) (s + d P s + d^2 P^2 s + d^3 P^3 s)              exact push
       + tm * w_i * m[a_i] / (sum_c m_c * cw[a_i])              learned tail

with a_i a k-means cluster of a seeded random-projection code of node i,
w = exp(two-layer message-passing network over log-degrees and the code),
m = relu(c K) the cluster masses predicted from the cluster mix c of
P^3 s and P^4 s.  K is fitted by least squares and the network by Adam, both
on PPR vectors the batched GPU solver computes.  The power iteration still
runs to the same tolerance from x0; a warm start whose first residual is not
below the cold start's is rejected and that set is solved again from s.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import struct
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native
from ._native import Config, Run, WarmConfig, WarmStats, ptr, score_buffer

PARAMS, COUPLING, CLUSTERS, FEATURES, CODE, WEIGHT = range(6)

# parameter layout of GOPS_WARM_PARAMS
W_IN, HIDDEN = 48, 128
P_W1 = 0
P_W2 = P_W1 + W_IN * HIDDEN
P_B2 = P_W2 + 2 * HIDDEN * HIDDEN
P_W3 = P_B2 + HIDDEN
P_B3 = P_W3 + HIDDEN
P_COUNT = P_B3 + 1


def default_config(**kw) -> WarmConfig:
    c = WarmConfig()
    _native.lib().gops_warm_config_default(ctypes.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise AttributeError(k)
        setattr(c, k, v)
    return c


# ---- checkpoint file: a trained model's parameters and cluster coupling ----
#
#   magic "GOPSWARM" | u32 version | u32 header length | header (UTF-8 JSON)
#   | payload: the arrays, little-endian, each starting on a 16-byte boundary
#
# The header holds the model's configuration, the graph's n, m and a SHA-256
# of its out-adjacency (row_ptr as int64, col as int32), and for each array
# its name, dtype, count and offset within the payload.  The clusters, the
# code and the features are not learned: a model created with the same
# configuration on the same graph rebuilds them (k-means is seeded), and the
# clusters are stored only to check that it did.

CHECKPOINT_MAGIC = b"GOPSWARM"
CHECKPOINT_VERSION = 1


def config_to_dict(cfg: WarmConfig) -> dict:
    return {name: getattr(cfg, name) for name, _ in cfg._fields_}


def config_from_dict(d: dict) -> WarmConfig:
    return default_config(**d)


def graph_digest(row_ptr, col) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(row_ptr, dtype="<i8").tobytes())
    h.update(np.ascontiguousarray(col, dtype="<i4").tobytes())
    return h.hexdigest()


def write_checkpoint(path, meta: dict, arrays: dict) -> None:
    """Writes meta (JSON-serialisable) and named 1-D arrays (float32 or int32)
    to path, through a temporary file renamed into place."""
    entries, blobs, off = [], [], 0
    for name, a in arrays.items():
        a = np.ascontiguousarray(a)
        dt = {np.dtype(np.float32): "<f4", np.dtype(np.int32): "<i4"}.get(a.dtype)
        if dt is None or a.ndim != 1:
            raise ValueError(f"array {name!r}: 1-D float32 or int32 expected")
        b = a.astype(dt).tobytes()
        entries.append({"name": name, "dtype": dt, "count": int(a.shape[0]), "offset": off})
        pad = (-len(b)) % 16
        blobs.append(b + b"\0" * pad)
        off += len(b) + pad
    head = json.dumps(dict(meta, arrays=entries), sort_keys=True).encode()
    pre = CHECKPOINT_MAGIC + struct.pack("<II", CHECKPOINT_VERSION, len(head)) + head
    pre += b"\0" * ((-len(pre)) % 16)
    tmp = f"{os.fspath(path)}.tmp"
    with open(tmp, "wb") as f:
        f.write(pre)
        for b in blobs:
            f.write(b)
    os.replace(tmp, path)


def read_checkpoint(path):
    """(meta, {name: array}) of a file written by write_checkpoint; raises
    ValueError for another format, another version or a truncated file."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 16 or data[:8] != CHECKPOINT_MAGIC:
        raise ValueError("not a warm-start checkpoint")
    version, hlen = struct.unpack_from("<II", data, 8)
    if version != CHECKPOINT_VERSION:
        raise ValueError(f"checkpoint version {version} is not supported (expected {CHECKPOINT_VERSION})")
    if 16 + hlen > len(data):
        raise ValueError("truncated checkpoint")
    try:
        meta = json.loads(data[16:16 + hlen].decode())
        entries = meta.pop("arrays")
    except (UnicodeDecodeError, json.JSONDecodeError, KeyError, AttributeError) as e:
        raise ValueError("corrupt checkpoint header") from e
    base = 16 + hlen + (-(16 + hlen)) % 16
    arrays = {}
    for e in entries:
        if e.get("dtype") not in ("<f4", "<i4"):
            raise ValueError("corrupt checkpoint header")
        dt = np.dtype(e["dtype"])
        lo = base + int(e["offset"])
        hi = lo + int(e["count"]) * dt.itemsize
        if lo < base or hi < lo or hi > len(data):
            raise ValueError("truncated checkpoint")
        arrays[e["name"]] = np.frombuffer(data[lo:hi], dtype=dt).astype(dt.newbyteorder("="))
    return meta, arrays


@dataclass
class LearnedRun:
    scores: Optional[np.ndarray]  # float32 [nsets, n], or None
    iterations: np.ndarray
    diff_l1: np.ndarray
    converged: np.ndarray
    rejected: np.ndarray          # warm start rejected, set solved again from s


def _cfg(cfg):
    return Config(float(cfg.damping), int(cfg.max_iterations), float(cfg.tolerance))


def _sets(seed_ptr, seed_idx):
    sp = np.ascontiguousarray(seed_ptr, dtype=np.int64)
    si = np.ascontiguousarray(seed_idx, dtype=np.int32)
    return sp, si, int(sp.shape[0]) - 1


class WarmStart:
    """A trained (or trainable) warm-start model bound to one DeviceGraph."""

    def __init__(self, graph: "_native.DeviceGraph", row_ptr, col, config: WarmConfig | None = None):
        self.graph = graph
        self.ctx = graph.ctx
        self.n = graph.n
        rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
        cc = np.ascontiguousarray(col, dtype=np.int32)
        cfg = config or default_config()
        h = _native._p()
        self.ctx.check(self.ctx._l.gops_warm_create(self.ctx.handle, graph.handle, ptr(rp), ptr(cc),
                                                     ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self.config = cfg
        self._rp, self._col = rp, cc  # for the graph digest of a checkpoint

    def save(self, path) -> None:
        """Writes the trained parameters and cluster coupling (and what a
        load checks them against) to a checkpoint file."""
        meta = {"config": config_to_dict(self.config), "n": int(self.n), "m": int(self._col.shape[0]),
                "graph_sha256": graph_digest(self._rp, self._col)}
        write_checkpoint(path, meta, {"params": self.get(PARAMS), "coupling": self.get(COUPLING),
                                      "clusters": self.get(CLUSTERS)})

    @classmethod
    def load(cls, path, graph: "_native.DeviceGraph", row_ptr, col) -> "WarmStart":
        """A model for graph with the parameters and coupling of a checkpoint.
        The graph must be the one the model was saved for (same out-adjacency);
        the model is rebuilt with the saved configuration and its clusters are
        checked against the saved ones before the parameters are set."""
        meta, arrays = read_checkpoint(path)
        rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
        cc = np.ascontiguousarray(col, dtype=np.int32)
        if (meta["n"] != rp.shape[0] - 1 or meta["m"] != cc.shape[0]
                or meta["graph_sha256"] != graph_digest(rp, cc)):
            raise ValueError("checkpoint was saved for a different graph")
        model = cls(graph, rp, cc, config_from_dict(meta["config"]))
        try:
            if not np.array_equal(model.get(CLUSTERS), arrays["clusters"]):
                raise ValueError("rebuilt clusters differ from the checkpoint's")
            model.set(PARAMS, arrays["params"])
            model.set(COUPLING, arrays["coupling"])
        except Exception:
            model.close()
            raise
        return model

    def close(self):
        if getattr(self, "handle", None):
            self.ctx._l.gops_warm_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def train(self, cfg, seed_ptr, seed_idx) -> WarmStats:
        sp, si, ns = _sets(seed_ptr, seed_idx)
        st = WarmStats()
        c = _cfg(cfg)
        self.ctx.check(self.ctx._l.gops_warm_train(self.ctx.handle, self.handle, ctypes.byref(c), ns,
                                                    ptr(sp), ptr(si), ctypes.byref(st)))
        return st

    def predict_device(self, damping, seed_ptr, seed_idx, x0_device_ptr: int):
        """Warm starts into a device buffer of nsets*n floats; returns r1_cold."""
        sp, si, ns = _sets(seed_ptr, seed_idx)
        r1 = np.empty(max(ns, 1), dtype=np.float64)
        self.ctx.check(self.ctx._l.gops_warm_predict(self.ctx.handle, self.handle, float(damping), ns, ptr(sp),
                                                      ptr(si), ctypes.c_void_p(x0_device_ptr), ptr(r1)))
        return r1[:ns]

    def ppr_batch(self, cfg, seed_ptr, seed_idx, scores=True) -> LearnedRun:
        """scores: True (a new array), False (none) or the caller's float32
        (nsets, n) array, as DeviceGraph.ppr_batch's out."""
        sp, si, ns = _sets(seed_ptr, seed_idx)
        c = _cfg(cfg)
        out = score_buffer(scores, ns, self.n)
        runs = (Run * max(ns, 1))()
        rej = np.zeros(max(ns, 1), dtype=np.int32)
        self.ctx.check(self.ctx._l.gops_ppr_batch_learned(self.ctx.handle, self.graph.handle, self.handle,
                                                           ctypes.byref(c), ns, ptr(sp), ptr(si), ptr(out),
                                                           ctypes.cast(runs, ctypes.c_void_p), ptr(rej)))
        its = np.array([runs[i].iterations for i in range(ns)], dtype=np.int64)
        diffs = np.array([runs[i].diff_l1 for i in range(ns)], dtype=np.float64)
        conv = np.array([bool(runs[i].converged) for i in range(ns)])
        return LearnedRun(out, its, diffs, conv, rej[:ns].astype(bool))

    def ppr_batch_device(self, cfg, seed_ptr, seed_idx, scores_device_ptr: int):
        """As ppr_batch with the scores left in a device buffer (nsets*n floats)."""
        sp, si, ns = _sets(seed_ptr, seed_idx)
        c = _cfg(cfg)
        runs = (Run * max(ns, 1))()
        rej = np.zeros(max(ns, 1), dtype=np.int32)
        self.ctx.check(self.ctx._l.gops_ppr_batch_learned_device(
            self.ctx.handle, self.graph.handle, self.handle, ctypes.byref(c), ns, ptr(sp), ptr(si),
            ctypes.c_void_p(scores_device_ptr), ctypes.cast(runs, ctypes.c_void_p), ptr(rej)))
        its = np.array([runs[i].iterations for i in range(ns)], dtype=np.int64)
        return its, rej[:ns].astype(bool)

    def get(self, what: int) -> np.ndarray:
        cnt = int(self.ctx._l.gops_warm_count(self.handle, what))
        dt = np.int32 if what == CLUSTERS else np.float32
        a = np.empty(max(cnt, 1), dtype=dt)
        self.ctx.check(self.ctx._l.gops_warm_get(self.ctx.handle, self.handle, what, ptr(a), cnt))
        return a[:cnt]

    def set(self, what: int, values) -> None:
        a = np.ascontiguousarray(values, dtype=np.float32).ravel()
        self.ctx.check(self.ctx._l.gops_warm_set(self.ctx.handle, self.handle, what, ptr(a), int(a.shape[0])))

    def loss_grad(self, damping, seed_ptr, seed_idx, targets_x):
        sp, si, ns = _sets(seed_ptr, seed_idx)
        t = np.ascontiguousarray(targets_x, dtype=np.float32)
        if t.shape != (ns, self.n):
            raise ValueError("targets_x must have shape (nsets, n)")
        loss = ctypes.c_double()
        g = np.empty(P_COUNT, dtype=np.float32)
        self.ctx.check(self.ctx._l.gops_warm_loss_grad(self.ctx.handle, self.handle, float(damping), ns, ptr(sp),
                                                        ptr(si), ptr(t), ctypes.byref(loss), ptr(g)))
        return loss.value, g

    def push(self, damping, seeds):
        s = np.ascontiguousarray(seeds, dtype=np.int32)
        r = int(self.ctx._l.gops_warm_count(self.handle, COUPLING))
        clusters = int(round((-1 + np.sqrt(1 + 8 * r)) / 4))  # (2c+1)c = r
        local = np.empty(self.n, dtype=np.float64)
        mix = np.empty(2 * clusters + 1, dtype=np.float64)
        tm, r1 = ctypes.c_double(), ctypes.c_double()
        self.ctx.check(self.ctx._l.gops_warm_push(self.ctx.handle, self.handle, float(damping), ptr(s),
                                                   int(s.shape[0]), ptr(local), ptr(mix), ctypes.byref(tm),
                                                   ctypes.byref(r1)))
        return local, mix, tm.value, r1.value
