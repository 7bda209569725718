"""top_k and normalize (src/topk.rs:17-61) on device-resident scores.

The host versions (``graphops_gb300.top_k``, ``normalize``) mirror the crate
for host arrays; these run on the GPU over CUDA pointers (for example the
scores of ``gops_ppr_batch_device``), so a caller can take the top entries of
each seed set without copying N x k score blocks to the host.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from ._native import ptr


def top_k_device(scores_ptr: int, n: int, k: int, ctx=None):
    """[(index, score)] of the k largest finite positive scores of a device
    FP64 vector, by score descending (ties by index)."""
    ctx = ctx or _native.default_context()
    idx = np.empty(max(k, 1), dtype=np.int64)
    val = np.empty(max(k, 1), dtype=np.float64)
    cnt = ctypes.c_int64(0)
    ctx.check(ctx._l.gops_top_k_f64_device(ctx.handle, ctypes.c_void_p(scores_ptr), int(n), int(k), ptr(idx),
                                           ptr(val), ctypes.byref(cnt)))
    return [(int(i), float(v)) for i, v in zip(idx[:cnt.value], val[:cnt.value])]


def top_k_rows_device(block_ptr: int, rows: int, n: int, k: int, ctx=None):
    """Per row of a device FP32 block (rows x n): (idx [rows, k], val [rows, k],
    counts [rows]); entries past counts[r] are unspecified."""
    ctx = ctx or _native.default_context()
    idx = np.empty((max(rows, 1), max(k, 1)), dtype=np.int64)
    val = np.empty((max(rows, 1), max(k, 1)), dtype=np.float32)
    cnt = np.zeros(max(rows, 1), dtype=np.int64)
    ctx.check(ctx._l.gops_top_k_f32_rows_device(ctx.handle, ctypes.c_void_p(block_ptr), int(rows), int(n), int(k),
                                                ptr(idx), ptr(val), ptr(cnt)))
    return idx[:rows, :k], val[:rows, :k], cnt[:rows]


def normalize_device(scores_ptr: int, n: int, ctx=None) -> None:
    """Divides a device FP64 vector by its sum when the sum is > 0."""
    ctx = ctx or _native.default_context()
    ctx.check(ctx._l.gops_normalize_f64_device(ctx.handle, ctypes.c_void_p(scores_ptr), int(n)))
