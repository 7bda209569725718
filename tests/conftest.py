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


def top_order_matches(a, b, k=100, tie=0.0):
    """True when the k largest entries of a come in the order of b's k
    largest, ties in b within 1e-15 relative counting as equal (the
    reference's top_k sorts by score with an unstable sort, src/topk.rs:40).
    `tie` (absolute) widens the ties for results that cannot order entries
    more finely than their own error: the FP32 score blocks of the batched
    path pass tie = 2 max|a - b|, so two entries may swap only when their
    reference scores differ by less than the result's largest error."""
    import numpy as np
    ia = np.argsort(-a, kind="stable")[:k]
    ib = np.argsort(-b, kind="stable")[:k]
    for x, y in zip(ia, ib):
        if x != y and abs(b[x] - b[y]) > max(1e-15 * max(abs(b[x]), 1e-300), tie):
            return False
    return True


def fp32_tie(a, b):
    """The tie width of top_order_matches for an FP32 result a against b."""
    import numpy as np
    return 2.0 * float(np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64)).max())


def sample_sets(sp, si, idx):
    """The seed sets idx of (seed_ptr, seed_idx) as a new (seed_ptr, seed_idx)."""
    import numpy as np
    lens = np.diff(sp)[idx]
    sp2 = np.zeros(len(idx) + 1, np.int64)
    sp2[1:] = np.cumsum(lens)
    si2 = np.concatenate([si[sp[i]:sp[i + 1]] for i in idx]).astype(np.int32) if len(idx) else np.zeros(0, np.int32)
    return sp2, si2
