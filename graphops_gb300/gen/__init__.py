"""Seeded synthetic graphs for the PageRank / PPR workloads (ctypes over
``libgraphgen.so``; the C source documents the generators).

Every generator returns a :class:`CsrGraph` holding the out-adjacency in the
order a graphops ``Graph`` adapter would list it (rows ascending, columns
ascending), with optional FP32 weights.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(os.path.dirname(_HERE), "libgraphgen.so")
_lib = None

_i64 = ctypes.c_int64
_p = ctypes.c_void_p


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise RuntimeError(f"{_LIB_PATH} is missing: run __graft_entry__.build() first")
    lib = ctypes.CDLL(_LIB_PATH)
    lib.gg_erdos_renyi.restype = _p
    lib.gg_erdos_renyi.argtypes = [_i64, ctypes.c_double, ctypes.c_double, ctypes.c_uint64]
    lib.gg_rmat.restype = _p
    lib.gg_rmat.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                            ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                            ctypes.c_uint64, ctypes.c_int]
    lib.gg_sbm.restype = _p
    lib.gg_sbm.argtypes = [_i64, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                           ctypes.c_double, ctypes.c_uint64, ctypes.c_int]
    lib.gg_n.restype = _i64
    lib.gg_n.argtypes = [_p]
    lib.gg_m.restype = _i64
    lib.gg_m.argtypes = [_p]
    lib.gg_weighted.restype = ctypes.c_int
    lib.gg_weighted.argtypes = [_p]
    lib.gg_export.restype = None
    lib.gg_export.argtypes = [_p, _p, _p, _p, _p]
    lib.gg_free.restype = None
    lib.gg_free.argtypes = [_p]
    lib.gg_seed_sets.restype = _i64
    lib.gg_seed_sets.argtypes = [_i64, _p, _i64, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_uint64, _p, _p]
    lib.gg_mix64.restype = ctypes.c_uint64
    lib.gg_mix64.argtypes = [ctypes.c_uint64]
    _lib = lib
    return lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class CsrGraph:
    """Out-adjacency CSR: row_ptr int64[n+1], col int32[m], weight f32[m] or None."""
    n: int
    row_ptr: np.ndarray
    col: np.ndarray
    weight: Optional[np.ndarray] = None
    block: Optional[np.ndarray] = None

    @property
    def m(self) -> int:
        return int(self.col.shape[0])

    def out_degree(self) -> np.ndarray:
        return np.diff(self.row_ptr)


def _take(h, want_block=False) -> CsrGraph:
    lib = _load()
    if not h:
        raise MemoryError("graph generator failed (allocation or bad arguments)")
    try:
        n, m = lib.gg_n(h), lib.gg_m(h)
        rp = np.empty(n + 1, dtype=np.int64)
        col = np.empty(m, dtype=np.int32)
        w = np.empty(m, dtype=np.float32) if lib.gg_weighted(h) else None
        blk = np.empty(n, dtype=np.int32) if want_block else None
        lib.gg_export(h, _ptr(rp), _ptr(col), _ptr(w), _ptr(blk))
    finally:
        lib.gg_free(h)
    return CsrGraph(n, rp, col, w, blk)


def _threads(threads):
    return threads if threads else max(1, min(64, os.cpu_count() or 1))


def erdos_renyi(n: int, p: float, dangling_frac: float = 0.0, seed: int = 0) -> CsrGraph:
    return _take(_load().gg_erdos_renyi(n, p, dangling_frac, seed))


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
         c: float = 0.19, weighted: bool = False, wlo: float = 0.1, whi: float = 1.0,
         seed: int = 0, threads: int = 0) -> CsrGraph:
    return _take(_load().gg_rmat(scale, edge_factor, a, b, c, int(weighted), wlo, whi,
                                 seed, _threads(threads)))


def sbm(n: int, blocks: int = 64, zipf_s: float = 1.2, intra_mean: float = 16.0,
        inter_mean: float = 4.0, seed: int = 0, threads: int = 0) -> CsrGraph:
    return _take(_load().gg_sbm(n, blocks, zipf_s, intra_mean, inter_mean, seed,
                                _threads(threads)), want_block=True)


def seed_sets(g: CsrGraph, nsets: int, lo: int, hi: int, seed: int = 0):
    """Returns (seed_ptr int64[nsets+1], seed_idx int32[total])."""
    lib = _load()
    sp = np.empty(nsets + 1, dtype=np.int64)
    si = np.empty(max(1, nsets * hi), dtype=np.int32)
    tot = lib.gg_seed_sets(g.n, _ptr(g.row_ptr), nsets, lo, hi, seed, _ptr(sp), _ptr(si))
    if tot < 0:
        raise ValueError("bad seed-set arguments")
    return sp, si[:tot].copy()


def dense_adjacency(g: CsrGraph) -> np.ndarray:
    """The n x n f64 matrix an AdjacencyMatrix caller would hold (1.0 or weight)."""
    M = np.zeros((g.n, g.n), dtype=np.float64)
    src = np.repeat(np.arange(g.n), np.diff(g.row_ptr))
    M[src, g.col] = 1.0 if g.weight is None else g.weight.astype(np.float64)
    return M
