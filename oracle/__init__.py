"""The oracle: CPU restatements of graphops' PageRank path, for checking only.

TEST INFRASTRUCTURE.  Only tests, the smoke check and the CPU-baseline leg of
the benchmark import this package; the product (graphops_gb300) never does.
"""
