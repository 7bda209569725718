import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the libgops kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Native pieces the tests load: the generator and oracle libraries always
    (plain gcc, cheap); libgops.so must already exist for GPU tests."""
    from graphops_gb300 import build as b
    b.build_graphgen()
    from oracle import build_oracle
    build_oracle.build()
    yield


def load_golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)["cases"]


def case_csr(c):
    import numpy as np
    nb = c["neighbors"]
    rp = np.zeros(len(nb) + 1, dtype=np.int64)
    for i, row in enumerate(nb):
        rp[i + 1] = rp[i] + len(row)
    col = np.array([v for row in nb for v in row], dtype=np.int32)
    w = None
    if c["weights"] is not None:
        w = np.array([x for row in c["weights"] for x in row], dtype=np.float64)
    return rp, col, w
