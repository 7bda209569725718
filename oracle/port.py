"""ctypes wrapper of the C restatement (pagerank_port.c -> liborcport.so).

TEST INFRASTRUCTURE ONLY (the oracle); see pagerank_port.c for the reference
lines each function follows.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


class OrcConfig(ctypes.Structure):
    _fields_ = [("damping", ctypes.c_double), ("max_iterations", ctypes.c_uint64),
                ("tolerance", ctypes.c_double)]


class OrcRun(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint64), ("diff_l1", ctypes.c_double),
                ("converged", ctypes.c_int32)]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.OUT
        if not os.path.exists(path):
            build_oracle.build()
        l = ctypes.CDLL(path)
        P = ctypes.c_void_p
        l.orc_pagerank_run.argtypes = [ctypes.c_int64, P, P, OrcConfig, P, ctypes.POINTER(OrcRun)]
        l.orc_pagerank_weighted_run.argtypes = [ctypes.c_int64, P, P, P, OrcConfig, P, ctypes.POINTER(OrcRun)]
        l.orc_ppr_run.argtypes = [ctypes.c_int64, P, P, P, OrcConfig, P, ctypes.POINTER(OrcRun)]
        l.orc_dense_to_csr.argtypes = [ctypes.c_int64, P, P, P, P, ctypes.c_int64]
        l.orc_dense_to_csr.restype = ctypes.c_int64
        l.orc_pagerank_run_dense.argtypes = [ctypes.c_int64, P, OrcConfig, P, ctypes.POINTER(OrcRun)]
        l.orc_ppr_many.argtypes = [ctypes.c_int64, P, P, OrcConfig, ctypes.c_int64, P, P,
                                   ctypes.c_int, P, P]
        l.orc_katz_run.argtypes = [ctypes.c_int64, P, P, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                   ctypes.c_double, P, ctypes.POINTER(OrcRun)]
        l.orc_hits_run.argtypes = [ctypes.c_int64, P, P, ctypes.c_uint64, ctypes.c_double, P, P,
                                   ctypes.POINTER(OrcRun)]
        l.orc_eigenvector_run.argtypes = [ctypes.c_int64, P, P, ctypes.c_uint64, ctypes.c_double, P,
                                          ctypes.POINTER(OrcRun)]
        l.orc_pagerank_weighted_run_mt.argtypes = [ctypes.c_int64, P, P, P, OrcConfig, ctypes.c_int, P,
                                                    ctypes.POINTER(OrcRun), ctypes.POINTER(ctypes.c_double)]
        _lib = l
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _cfg(damping, max_iterations, tolerance):
    return OrcConfig(float(damping), int(max_iterations), float(tolerance))


def pagerank_run(row_ptr, col, damping=0.85, max_iterations=100, tolerance=1e-6):
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    n = rp.shape[0] - 1
    out = np.empty(max(n, 1))
    r = OrcRun()
    if lib().orc_pagerank_run(n, _p(rp), _p(cl), _cfg(damping, max_iterations, tolerance), _p(out), ctypes.byref(r)):
        raise MemoryError
    return out[:n], int(r.iterations), float(r.diff_l1), bool(r.converged)


def pagerank_weighted_run(row_ptr, col, w, damping=0.85, max_iterations=100, tolerance=1e-6):
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    ww = np.ascontiguousarray(w, dtype=np.float64)
    n = rp.shape[0] - 1
    out = np.empty(max(n, 1))
    r = OrcRun()
    if lib().orc_pagerank_weighted_run(n, _p(rp), _p(cl), _p(ww), _cfg(damping, max_iterations, tolerance), _p(out), ctypes.byref(r)):
        raise MemoryError
    return out[:n], int(r.iterations), float(r.diff_l1), bool(r.converged)


def ppr_run(row_ptr, col, p, damping=0.85, max_iterations=100, tolerance=1e-6):
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    pp = np.ascontiguousarray(p, dtype=np.float64)
    n = rp.shape[0] - 1
    out = np.empty(max(n, 1))
    r = OrcRun()
    if lib().orc_ppr_run(n, _p(rp), _p(cl), _p(pp), _cfg(damping, max_iterations, tolerance), _p(out), ctypes.byref(r)):
        raise MemoryError
    return out[:n], int(r.iterations), float(r.diff_l1), bool(r.converged)


def dense_to_csr(M):
    M = np.ascontiguousarray(M, dtype=np.float64)
    n = M.shape[0]
    cap = int(np.count_nonzero(M > 0.0))
    rp = np.empty(n + 1, dtype=np.int64)
    cl = np.empty(max(cap, 1), dtype=np.int32)
    w = np.empty(max(cap, 1), dtype=np.float64)
    m = lib().orc_dense_to_csr(n, _p(M), _p(rp), _p(cl), _p(w), cap)
    return rp, cl[:m], w[:m]


def pagerank_run_dense(M, damping=0.85, max_iterations=100, tolerance=1e-6):
    M = np.ascontiguousarray(M, dtype=np.float64)
    n = M.shape[0]
    out = np.empty(max(n, 1))
    r = OrcRun()
    if lib().orc_pagerank_run_dense(n, _p(M), _cfg(damping, max_iterations, tolerance), _p(out), ctypes.byref(r)):
        raise MemoryError
    return out[:n], int(r.iterations), float(r.diff_l1), bool(r.converged)


def ppr_many(row_ptr, col, seed_ptr, seed_idx, damping=0.85, max_iterations=100,
             tolerance=1e-6, threads=1, want_scores=True):
    """One reference PPR solve per seed set (p = 1 per occurrence of each
    seed, so a repeated node counts twice); returns
    (scores[nsets, n] or None, iterations[nsets])."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    sp = np.ascontiguousarray(seed_ptr, dtype=np.int64)
    si = np.ascontiguousarray(seed_idx, dtype=np.int32)
    n = rp.shape[0] - 1
    ns = sp.shape[0] - 1
    out = np.empty((ns, n)) if want_scores else None
    its = np.zeros(ns, dtype=np.uint64)
    if lib().orc_ppr_many(n, _p(rp), _p(cl), _cfg(damping, max_iterations, tolerance), ns,
                          _p(sp), _p(si), int(threads), _p(out), _p(its)):
        raise MemoryError
    return out, its


def katz_run(row_ptr, col, alpha=0.1, beta=1.0, max_iterations=100, tolerance=1e-6):
    """katz_centrality_run (src/katz.rs:136-201) in FP64."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    n = rp.shape[0] - 1
    out = np.empty(max(n, 1))
    r = OrcRun()
    if lib().orc_katz_run(n, _p(rp), _p(cl), float(alpha), float(beta), int(max_iterations), float(tolerance),
                          _p(out), ctypes.byref(r)):
        raise MemoryError
    return out[:n], int(r.iterations), float(r.diff_l1), bool(r.converged)


def eigenvector_run(row_ptr, col, max_iterations=100, tolerance=1e-6):
    """eigenvector_centrality_run (src/eigenvector.rs:49-125) in FP64."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    n = rp.shape[0] - 1
    out = np.empty(max(n, 1))
    r = OrcRun()
    if lib().orc_eigenvector_run(n, _p(rp), _p(cl), int(max_iterations), float(tolerance), _p(out),
                                 ctypes.byref(r)):
        raise MemoryError
    return out[:n], int(r.iterations), float(r.diff_l1), bool(r.converged)


def hits_run(row_ptr, col, max_iterations=100, tolerance=1e-6):
    """hits (src/centrality.rs:114-166) in FP64: (hub, auth, iterations, last L2 change, converged)."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    n = rp.shape[0] - 1
    hub = np.empty(max(n, 1))
    auth = np.empty(max(n, 1))
    r = OrcRun()
    if lib().orc_hits_run(n, _p(rp), _p(cl), int(max_iterations), float(tolerance), _p(hub), _p(auth),
                          ctypes.byref(r)):
        raise MemoryError
    return hub[:n], auth[:n], int(r.iterations), float(r.diff_l1), bool(r.converged)


def pagerank_weighted_run_mt(row_ptr, col, w, damping=0.85, max_iterations=100, tolerance=1e-6, threads=1):
    """All-cores timing form of pagerank_weighted_run (pull over an in-CSR,
    rows split over `threads` host threads; a CPU baseline, not a parity
    reference).  Returns (scores, iterations, diff_l1, converged, seconds of
    the iterations alone)."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    w = np.ascontiguousarray(w, dtype=np.float64)
    n = row_ptr.shape[0] - 1
    out = np.empty(max(n, 1))
    r = OrcRun()
    secs = ctypes.c_double()
    if lib().orc_pagerank_weighted_run_mt(n, _p(row_ptr), _p(col), _p(w), _cfg(damping, max_iterations, tolerance),
                                          int(threads), _p(out), ctypes.byref(r), ctypes.byref(secs)):
        raise MemoryError
    return out[:n], int(r.iterations), float(r.diff_l1), bool(r.converged), float(secs.value)
