"""ctypes bindings of libgops.so (the C ABI in include/gops.h).

The library is required: importing the operators without it raises, and there
is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# GOPS_LIBRARY may name another build of the same ABI (e.g. one compiled with
# different tuning macros); by default the in-tree build is loaded.
LIB_PATH = os.environ.get("GOPS_LIBRARY") or os.path.join(_HERE, "libgops.so")

GOPS_OK = 0
GOPS_ERR_INVALID = 1
GOPS_ERR_OOM = 2
GOPS_ERR_CUDA = 3
GOPS_ERR_TIMEOUT = 4
GOPS_ERR_NO_DEVICE = 5
GOPS_ERR_INTERNAL = 6

_p = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64
_dbl = ctypes.c_double


class Config(ctypes.Structure):
    _fields_ = [("damping", _dbl), ("max_iterations", _u64), ("tolerance", _dbl)]


class Run(ctypes.Structure):
    _fields_ = [("iterations", _u64), ("diff_l1", _dbl), ("converged", _i32), ("reserved", _i32)]


class Stats(ctypes.Structure):
    _fields_ = [("solve_ms", _dbl), ("iterate_ms", _dbl), ("kernel_launches", _u64),
                ("iterations", _u64), ("h2d_bytes", _u64), ("d2h_bytes", _u64),
                ("df_ms", _dbl), ("df_launches", _u64), ("f32_ms", _dbl), ("f32_launches", _u64)]


class KatzConfig(ctypes.Structure):
    _fields_ = [("alpha", _dbl), ("beta", _dbl), ("max_iterations", _u64), ("tolerance", _dbl)]


class WarmConfig(ctypes.Structure):
    _fields_ = [("clusters", _i32), ("code_steps", _i32), ("kmeans_iters", _i32), ("minibatch", _i32),
                ("chunk", _i32), ("epochs", _i32), ("lr", ctypes.c_float), ("ridge", ctypes.c_float),
                ("seed", _u64), ("push_budget", _i64)]


class WarmStats(ctypes.Structure):
    _fields_ = [("loss_first", _dbl), ("loss_last", _dbl), ("steps", _i64), ("sets", _i64),
                ("target_ms", _dbl), ("fit_ms", _dbl)]


# (name, restype, argtypes) for every symbol include/gops.h declares
SIGNATURES = [
    ("gops_abi_version", ctypes.c_int, []),
    ("gops_debug_fail_allocations_after", ctypes.c_int, [ctypes.c_int64]),
    ("gops_debug_tc_gemm", ctypes.c_int, [_p, ctypes.c_int, _p, _p, _p, _i64, _p, _p, _p, _p, _p]),
    ("gops_ctx_create", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_p)]),
    ("gops_ctx_destroy", None, [_p]),
    ("gops_last_error", ctypes.c_char_p, [_p]),
    ("gops_ctx_stats", ctypes.c_int, [_p, ctypes.POINTER(Stats)]),
    ("gops_ctx_stream", _p, [_p]),
    ("gops_ctx_set_timing", ctypes.c_int, [_p, ctypes.c_int]),
    ("gops_config_validate", ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_char_p, ctypes.c_size_t]),
    ("gops_weights_validate", ctypes.c_int, [_i64, _p, ctypes.c_char_p, ctypes.c_size_t]),
    ("gops_personalization_validate", ctypes.c_int, [_i64, _i64, _p, ctypes.c_char_p, ctypes.c_size_t]),
    ("gops_graph_upload", ctypes.c_int, [_p, _i64, _p, _p, _p, ctypes.POINTER(_p)]),
    ("gops_graph_from_dense", ctypes.c_int, [_p, _i64, _p, ctypes.POINTER(_p)]),
    ("gops_graph_from_edges", ctypes.c_int, [_p, _i64, _i64, _p, _p, _p, ctypes.POINTER(_p)]),
    ("gops_graph_destroy", None, [_p]),
    ("gops_graph_info", ctypes.c_int, [_p, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i32)]),
    ("gops_pagerank_run", ctypes.c_int, [_p, _p, ctypes.POINTER(Config), _p, ctypes.POINTER(Run)]),
    ("gops_pagerank_weighted_run", ctypes.c_int, [_p, _p, ctypes.POINTER(Config), _p, ctypes.POINTER(Run)]),
    ("gops_personalized_pagerank_run", ctypes.c_int, [_p, _p, ctypes.POINTER(Config), _p, _p, ctypes.POINTER(Run)]),
    ("gops_ctx_scores_device", _p, [_p]),
    ("gops_pagerank_run_noalloc", ctypes.c_int, [_p, _p, ctypes.POINTER(Config), _p, ctypes.POINTER(Run)]),
    ("gops_ppr_batch", ctypes.c_int, [_p, _p, ctypes.POINTER(Config), _i64, _p, _p, _p, _p, _p]),
    ("gops_ppr_batch_device", ctypes.c_int, [_p, _p, ctypes.POINTER(Config), _i64, _p, _p, _p, _p, _p]),
    ("gops_ppr_batch_set_tile", ctypes.c_int, [_p, _p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    ("gops_ppr_batch_tile", ctypes.c_int, [_p, _p, _p, _p, _p]),
    ("gops_katz_config_validate", ctypes.c_int, [ctypes.POINTER(KatzConfig), ctypes.c_char_p, ctypes.c_size_t]),
    ("gops_katz_run", ctypes.c_int, [_p, _p, ctypes.POINTER(KatzConfig), _p, ctypes.POINTER(Run)]),
    ("gops_eigenvector_run", ctypes.c_int, [_p, _p, _u64, _dbl, _p, ctypes.POINTER(Run)]),
    ("gops_hits_run", ctypes.c_int, [_p, _p, _u64, _dbl, _p, _p, ctypes.POINTER(Run)]),
    ("gops_top_k_f64_device", ctypes.c_int, [_p, _p, _i64, _i64, _p, _p, ctypes.POINTER(_i64)]),
    ("gops_top_k_f32_rows_device", ctypes.c_int, [_p, _p, _i64, _i64, _i64, _p, _p, _p]),
    ("gops_normalize_f64_device", ctypes.c_int, [_p, _p, _i64]),
    ("gops_warm_config_default", None, [ctypes.POINTER(WarmConfig)]),
    ("gops_warm_create", ctypes.c_int, [_p, _p, _p, _p, ctypes.POINTER(WarmConfig), ctypes.POINTER(_p)]),
    ("gops_warm_destroy", None, [_p]),
    ("gops_warm_train", ctypes.c_int, [_p, _p, ctypes.POINTER(Config), _i64, _p, _p, ctypes.POINTER(WarmStats)]),
    ("gops_warm_predict", ctypes.c_int, [_p, _p, _dbl, _i64, _p, _p, _p, _p]),
    ("gops_ppr_batch_learned", ctypes.c_int, [_p, _p, _p, ctypes.POINTER(Config), _i64, _p, _p, _p, _p, _p]),
    ("gops_ppr_batch_learned_device", ctypes.c_int,
     [_p, _p, _p, ctypes.POINTER(Config), _i64, _p, _p, _p, _p, _p]),
    ("gops_ppr_batch_judged_device", ctypes.c_int,
     [_p, _p, ctypes.POINTER(Config), _i64, _p, _p, _p, _p, _p, _p, _p]),
    ("gops_warm_count", _i64, [_p, ctypes.c_int]),
    ("gops_warm_get", ctypes.c_int, [_p, _p, ctypes.c_int, _p, _i64]),
    ("gops_warm_set", ctypes.c_int, [_p, _p, ctypes.c_int, _p, _i64]),
    ("gops_warm_loss_grad", ctypes.c_int, [_p, _p, _dbl, _i64, _p, _p, _p, ctypes.POINTER(_dbl), _p]),
    ("gops_warm_push", ctypes.c_int, [_p, _p, _dbl, _p, _i64, _p, _p, ctypes.POINTER(_dbl), ctypes.POINTER(_dbl)]),
]

_lib = None
_lock = threading.Lock()


def lib():
    """The loaded libgops.so; raises when it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: the CUDA library must be built "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        l = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class GopsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libgops error {code}: {msg}")
        self.code = code


class Context:
    """A gops_ctx: one CUDA device, one stream.  Use from one thread at a time."""

    def __init__(self, device: int = 0):
        self._l = lib()
        h = _p()
        rc = self._l.gops_ctx_create(device, ctypes.byref(h))
        if rc != GOPS_OK:
            raise GopsError(rc, "gops_ctx_create failed (no usable CUDA device?)")
        self.handle = h
        self.device = device

    def check(self, rc):
        if rc != GOPS_OK:
            raise GopsError(rc, self._l.gops_last_error(self.handle).decode())

    def stats(self) -> Stats:
        s = Stats()
        self.check(self._l.gops_ctx_stats(self.handle, ctypes.byref(s)))
        return s

    def set_timing(self, enable: bool) -> None:
        self.check(self._l.gops_ctx_set_timing(self.handle, int(bool(enable))))

    def stream(self) -> int:
        return self._l.gops_ctx_stream(self.handle) or 0

    def close(self):
        if getattr(self, "handle", None):
            self._l.gops_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def default_context() -> Context:
    """A lazily created context per host thread on device 0."""
    c = getattr(_tls, "ctx", None)
    if c is None:
        c = Context(int(os.environ.get("GOPS_DEVICE", "0")))
        _tls.ctx = c
    return c


def score_buffer(out, nsets: int, n: int):
    """The batched calls' score destination: out=True a new array, False
    none, or the caller's own array (checked: float32, C-contiguous,
    shape (nsets, n))."""
    if isinstance(out, np.ndarray):
        if out.dtype != np.float32 or out.shape != (nsets, n) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float32 array of shape (nsets, n)")
        return out
    return np.empty((nsets, n), dtype=np.float32) if out else None


class DeviceGraph:
    """A graph resident on the device (a gops_graph)."""

    def __init__(self, ctx: Context, handle, n: int, m: int, weighted: bool):
        self.ctx, self.handle, self.n, self.m, self.weighted = ctx, handle, n, m, weighted

    @classmethod
    def from_csr(cls, row_ptr, col, weights=None, ctx: Context | None = None):
        ctx = ctx or default_context()
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.int32)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        n = int(row_ptr.shape[0]) - 1
        if w is not None and w.shape[0] != col.shape[0]:
            raise ValueError("weights and col differ in length")
        h = _p()
        ctx.check(ctx._l.gops_graph_upload(ctx.handle, n, ptr(row_ptr), ptr(col), ptr(w), ctypes.byref(h)))
        return cls(ctx, h, n, int(col.shape[0]), w is not None)

    @classmethod
    def from_dense(cls, matrix, ctx: Context | None = None):
        ctx = ctx or default_context()
        M = np.ascontiguousarray(matrix, dtype=np.float64)
        n = int(M.shape[0]) if M.ndim == 2 else 0
        if M.ndim != 2 or M.shape[0] != M.shape[1]:
            raise ValueError("adjacency matrix must be square")
        h = _p()
        ctx.check(ctx._l.gops_graph_from_dense(ctx.handle, n, ptr(M), ctypes.byref(h)))
        nn, mm, ww = _i64(), _i64(), _i32()
        ctx._l.gops_graph_info(h, ctypes.byref(nn), ctypes.byref(mm), ctypes.byref(ww))
        return cls(ctx, h, nn.value, mm.value, bool(ww.value))

    @classmethod
    def from_edges(cls, n, src, dst, weights=None, ctx: Context | None = None):
        """A petgraph-style raw edge list (edge e: src[e] -> dst[e], in edge
        order) built on the device into the adapter's out-adjacency: rows
        newest edge first, each parallel u->v entry weighted like the newest."""
        ctx = ctx or default_context()
        s = np.ascontiguousarray(src, dtype=np.int32)
        d = np.ascontiguousarray(dst, dtype=np.int32)
        if s.shape != d.shape:
            raise ValueError("src and dst must have the same length")
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
        if w is not None and w.shape != s.shape:
            raise ValueError("weights must have one entry per edge")
        h = _p()
        ctx.check(ctx._l.gops_graph_from_edges(ctx.handle, int(n), int(s.shape[0]), ptr(s), ptr(d), ptr(w),
                                               ctypes.byref(h)))
        nn, mm, ww = _i64(), _i64(), _i32()
        ctx._l.gops_graph_info(h, ctypes.byref(nn), ctypes.byref(mm), ctypes.byref(ww))
        return cls(ctx, h, nn.value, mm.value, bool(ww.value))

    def close(self):
        if getattr(self, "handle", None):
            self.ctx._l.gops_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _solve(self, fn_name, cfg, p=None, out=True):
        c = Config(float(cfg.damping), int(cfg.max_iterations), float(cfg.tolerance))
        r = Run()
        scores = np.empty(self.n, dtype=np.float64) if out else None
        fn = getattr(self.ctx._l, fn_name)
        if p is None:
            rc = fn(self.ctx.handle, self.handle, ctypes.byref(c), ptr(scores), ctypes.byref(r))
        else:
            pp = np.ascontiguousarray(p, dtype=np.float64)
            rc = fn(self.ctx.handle, self.handle, ctypes.byref(c), ptr(pp), ptr(scores), ctypes.byref(r))
        self.ctx.check(rc)
        return scores, int(r.iterations), float(r.diff_l1), bool(r.converged)

    def ppr_batch(self, cfg, seed_ptr, seed_idx, x0=None, out=True):
        """Batched PPR over seed sets (CSR: seed_ptr[nsets+1], seed_idx).
        out: True (a new array), False (no scores) or the caller's C-contiguous
        float32 array of shape (nsets, n), e.g. a page-locked one, which the
        library fills by DMA without staging.
        Returns (scores float32 [nsets, n] or None, iterations, diff_l1, converged)."""
        sp = np.ascontiguousarray(seed_ptr, dtype=np.int64)
        si = np.ascontiguousarray(seed_idx, dtype=np.int32)
        ns = int(sp.shape[0]) - 1
        c = Config(float(cfg.damping), int(cfg.max_iterations), float(cfg.tolerance))
        scores = score_buffer(out, ns, self.n)
        xx = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float32)
        if xx is not None and xx.shape != (ns, self.n):
            raise ValueError("x0 must have shape (nsets, n)")
        runs = (Run * max(ns, 1))()
        self.ctx.check(self.ctx._l.gops_ppr_batch(self.ctx.handle, self.handle, ctypes.byref(c), ns,
                                                  ptr(sp), ptr(si), ptr(xx), ptr(scores),
                                                  ctypes.cast(runs, ctypes.c_void_p)))
        its = np.array([runs[i].iterations for i in range(ns)], dtype=np.int64)
        diffs = np.array([runs[i].diff_l1 for i in range(ns)], dtype=np.float64)
        conv = np.array([bool(runs[i].converged) for i in range(ns)])
        return scores, its, diffs, conv

    def set_batch_tile(self, cols=0, chunk=256, l2_hints=False):
        """Fix the batched path's k-tile (sets per wave: 32, 64 or 128), the
        chunk size of long rows and the FP32 step's L2 hints, or re-run the
        autotuner (cols=0)."""
        self.ctx.check(self.ctx._l.gops_ppr_batch_set_tile(self.ctx.handle, self.handle, int(cols), int(chunk),
                                                           int(bool(l2_hints))))

    def batch_tile(self):
        """(cols, chunk, l2_hints, cost) of the batched path: cost[i, j] is
        the autotuner's ms per set-step for cols 32/64/128 (i) and chunk
        256/1024 (j) without L2 hints, cost_l2 that of the chosen tile with
        them; 0 where not tried."""
        c, ch, l2 = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        cost = np.zeros(7, dtype=np.float32)
        self.ctx.check(self.ctx._l.gops_ppr_batch_tile(self.handle, ctypes.byref(c), ctypes.byref(ch),
                                                       ctypes.byref(l2), ptr(cost)))
        return int(c.value), int(ch.value), bool(l2.value), cost[:6].reshape(3, 2), float(cost[6])

    def katz_run(self, alpha, beta, max_iterations, tolerance, out=True):
        c = KatzConfig(float(alpha), float(beta), int(max_iterations), float(tolerance))
        r = Run()
        scores = np.empty(self.n, dtype=np.float64) if out else None
        self.ctx.check(self.ctx._l.gops_katz_run(self.ctx.handle, self.handle, ctypes.byref(c), ptr(scores),
                                                 ctypes.byref(r)))
        return scores, int(r.iterations), float(r.diff_l1), bool(r.converged)

    def eigenvector_run(self, max_iterations, tolerance, out=True):
        r = Run()
        scores = np.empty(self.n, dtype=np.float64) if out else None
        self.ctx.check(self.ctx._l.gops_eigenvector_run(self.ctx.handle, self.handle, int(max_iterations),
                                                        float(tolerance), ptr(scores), ctypes.byref(r)))
        return scores, int(r.iterations), float(r.diff_l1), bool(r.converged)

    def hits_run(self, max_iterations, tolerance):
        r = Run()
        hub = np.empty(self.n, dtype=np.float64)
        auth = np.empty(self.n, dtype=np.float64)
        self.ctx.check(self.ctx._l.gops_hits_run(self.ctx.handle, self.handle, int(max_iterations),
                                                 float(tolerance), ptr(hub), ptr(auth), ctypes.byref(r)))
        return hub, auth, int(r.iterations), float(r.diff_l1), bool(r.converged)

    def pagerank_run(self, cfg, out=True):
        return self._solve("gops_pagerank_run", cfg, out=out)

    def pagerank_weighted_run(self, cfg, out=True):
        return self._solve("gops_pagerank_weighted_run", cfg, out=out)

    def personalized_pagerank_run(self, cfg, p, out=True):
        return self._solve("gops_personalized_pagerank_run", cfg, p=p, out=out)
