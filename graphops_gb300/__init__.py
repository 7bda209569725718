"""graphops_gb300: graphops' PageRank / personalized-PageRank path on GB300.

The public names mirror the reference crate's (graphops 0.4.1, src/lib.rs:
47-48, 77-88): ``pagerank``, ``pagerank_run``, ``pagerank_checked``,
``pagerank_checked_run``, ``pagerank_weighted`` (+ ``_run``, ``_checked``,
``_checked_run``), ``personalized_pagerank`` (+ variants), ``PageRankConfig``,
``PageRankRun`` and the graph adapters.  The computation runs in libgops.so
(include/gops.h), CUDA for sm_103a; there is no CPU code path.
"""
from .graph import AdjacencyMatrix, CsrAdjacency, DiGraph
from .pagerank import (
    GraphopsError,
    InvalidParameter,
    PageRankConfig,
    PageRankRun,
    normalize,
    pagerank,
    pagerank_checked,
    pagerank_checked_run,
    pagerank_run,
    pagerank_weighted,
    pagerank_weighted_checked,
    pagerank_weighted_checked_run,
    pagerank_weighted_run,
    personalized_pagerank,
    personalized_pagerank_checked,
    personalized_pagerank_checked_run,
    personalized_pagerank_run,
    top_k,
)
from ._native import Context, DeviceGraph, GopsError, default_context
from .batch import BatchRun, ppr_batch, seed_sets_to_csr
from .centrality import (EigenvectorRun, KatzConfig, KatzRun, eigenvector_centrality,
                         eigenvector_centrality_run, hits, katz_centrality, katz_centrality_checked,
                         katz_centrality_run)

__all__ = [
    "AdjacencyMatrix", "CsrAdjacency", "DiGraph", "GraphopsError", "InvalidParameter",
    "PageRankConfig", "PageRankRun", "normalize", "pagerank", "pagerank_checked",
    "pagerank_checked_run", "pagerank_run", "pagerank_weighted", "pagerank_weighted_checked",
    "pagerank_weighted_checked_run", "pagerank_weighted_run", "personalized_pagerank",
    "personalized_pagerank_checked", "personalized_pagerank_checked_run",
    "personalized_pagerank_run", "top_k", "Context", "DeviceGraph", "GopsError",
    "default_context", "BatchRun", "ppr_batch", "seed_sets_to_csr", "KatzConfig", "KatzRun",
    "EigenvectorRun", "katz_centrality", "katz_centrality_run", "katz_centrality_checked",
    "eigenvector_centrality", "eigenvector_centrality_run", "hits",
]
