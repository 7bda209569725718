"""Katz, eigenvector and HITS centrality: the same pull power iteration as
PageRank, on the GPU, with the reference crate's names, defaults, messages
and diagnostics (graphops 0.4.1, src/katz.rs and src/eigenvector.rs).

Both take any graph adapter (``neighbors(u)`` out-lists; weights ignored), an
``AdjacencyMatrix``, or a ``DeviceGraph`` already on the device.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native
from .pagerank import InvalidParameter, _device_graph, _n


@dataclass
class KatzConfig:
    """KatzConfig (src/katz.rs:19-57): alpha 0.1, beta 1.0, 100 iterations, tol 1e-6."""
    alpha: float = 0.1
    beta: float = 1.0
    max_iterations: int = 100
    tolerance: float = 1e-6

    def validate(self) -> None:
        """src/katz.rs:60-86, the library's gops_katz_config_validate."""
        if isinstance(self.max_iterations, int) and self.max_iterations < 0:
            raise InvalidParameter("max_iterations must be > 0")
        c = _native.KatzConfig(float(self.alpha), float(self.beta), int(self.max_iterations), float(self.tolerance))
        buf = ctypes.create_string_buffer(256)
        if _native.lib().gops_katz_config_validate(ctypes.byref(c), buf, 256) != 0:
            raise InvalidParameter(buf.value.decode())


@dataclass
class KatzRun:
    """KatzRun (src/katz.rs:95-108)."""
    scores: np.ndarray
    iterations: int
    diff_l1: float
    converged: bool


@dataclass
class EigenvectorRun:
    """EigenvectorRun (src/eigenvector.rs:13-23)."""
    scores: np.ndarray
    iterations: int
    diff_l1: float
    converged: bool


def katz_centrality_run(graph, config: KatzConfig = None) -> KatzRun:
    """katz_centrality_run (src/katz.rs:136-201)."""
    config = config or KatzConfig()
    if _n(graph) == 0:
        return KatzRun(np.empty(0), 0, 0.0, True)
    dg = _device_graph(graph, weighted=False)
    s, it, diff, conv = dg.katz_run(config.alpha, config.beta, config.max_iterations, config.tolerance)
    return KatzRun(s, it, diff, conv)


def katz_centrality(graph, config: KatzConfig = None) -> np.ndarray:
    """katz_centrality (src/katz.rs:131-133)."""
    return katz_centrality_run(graph, config).scores


def katz_centrality_checked(graph, config: KatzConfig = None) -> np.ndarray:
    """katz_centrality_checked (src/katz.rs:207-210): validate, then run."""
    config = config or KatzConfig()
    config.validate()
    return katz_centrality(graph, config)


def eigenvector_centrality_run(graph, max_iterations: int = 100, tolerance: float = 1e-6) -> EigenvectorRun:
    """eigenvector_centrality_run (src/eigenvector.rs:49-125)."""
    if _n(graph) == 0:
        return EigenvectorRun(np.empty(0), 0, 0.0, True)
    dg = _device_graph(graph, weighted=False)
    s, it, diff, conv = dg.eigenvector_run(max_iterations, tolerance)
    return EigenvectorRun(s, it, diff, conv)


def eigenvector_centrality(graph) -> np.ndarray:
    """eigenvector_centrality (src/eigenvector.rs:26-28): 100 iterations, tol 1e-6."""
    return eigenvector_centrality_run(graph, 100, 1e-6).scores


def hits(graph, max_iter: int = 100, tol: float = 1e-6):
    """hits (src/centrality.rs:114-166): (hub scores, authority scores)."""
    if _n(graph) == 0:
        return np.empty(0), np.empty(0)
    dg = _device_graph(graph, weighted=False)
    hub, auth, _, _, _ = dg.hits_run(max_iter, tol)
    return hub, auth
