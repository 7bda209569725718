"""Host-side helpers of the batched and learned paths and the test hook,
callable without a device: the CSR form of seed sets, the warm-start
defaults, Katz validation messages through the library, and the allocation
fault hook's switch."""
import ctypes
import math

import numpy as np
import pytest

import graphops_gb300 as go
from graphops_gb300 import _native, warm


def test_seed_sets_to_csr():
    sp, si = go.seed_sets_to_csr([[3, 1], [], [7, 7, 2]])
    assert sp.tolist() == [0, 2, 2, 5] and si.tolist() == [3, 1, 7, 7, 2]
    assert sp.dtype == np.int64 and si.dtype == np.int32
    sp0, si0 = go.seed_sets_to_csr([])
    assert sp0.tolist() == [0] and si0.size == 0


def test_warm_defaults_and_overrides():
    c = warm.default_config()
    assert c.clusters == 128 and c.code_steps == 10 and c.kmeans_iters == 20
    assert c.minibatch == 32 and c.chunk == 512 and c.epochs == 1
    assert c.push_budget == 1 << 24 and c.lr > 0 and c.ridge >= 0
    c2 = warm.default_config(clusters=72, seed=5)
    assert c2.clusters == 72 and c2.seed == 5
    with pytest.raises(AttributeError):
        warm.default_config(no_such_field=1)


@pytest.mark.parametrize("kw,msg", [
    (dict(alpha=0.0), "alpha must be finite and > 0"),
    (dict(alpha=math.nan), "alpha must be finite and > 0"),
    (dict(beta=math.inf), "beta must be finite"),
    (dict(tolerance=0.0), "tolerance must be finite and > 0"),
])
def test_katz_validate_messages(kw, msg):
    with pytest.raises(go.InvalidParameter, match=msg):
        go.KatzConfig(**kw).validate()


def test_allocation_fault_hook_switch():
    lib = _native.lib()
    assert lib.gops_debug_fail_allocations_after(ctypes.c_int64(5)) == 0
    assert lib.gops_debug_fail_allocations_after(ctypes.c_int64(-1)) == 0


NULL_EXEMPT = {
    # no context argument, or a value-returning query with its own null answer
    "gops_abi_version", "gops_debug_fail_allocations_after", "gops_ctx_create", "gops_config_validate",
    "gops_weights_validate", "gops_personalization_validate", "gops_katz_config_validate",
    "gops_warm_config_default", "gops_ctx_destroy", "gops_graph_destroy", "gops_warm_destroy",
    "gops_last_error", "gops_ctx_stream", "gops_ctx_scores_device", "gops_warm_count",
}


def null_args(argtypes):
    out = []
    for t in argtypes:
        if t in (ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_size_t):
            out.append(t(0))
        elif t is ctypes.c_double:
            out.append(0.5)
        else:
            out.append(None)
    return out


@pytest.mark.parametrize("name", sorted(n for n, r, _ in _native.SIGNATURES if n not in NULL_EXEMPT))
def test_every_entry_point_rejects_a_null_context(name):
    """A NULL context (and NULL everything else) is GOPS_ERR_INVALID before
    any device call, for every status-returning entry point."""
    lib = _native.lib()
    fn = getattr(lib, name)
    assert fn(*null_args(fn.argtypes)) == _native.GOPS_ERR_INVALID, name


def test_null_queries_and_destroys_are_safe():
    lib = _native.lib()
    lib.gops_ctx_destroy(None)
    lib.gops_graph_destroy(None)
    lib.gops_warm_destroy(None)
    assert lib.gops_last_error(None) == b"null context"
    assert lib.gops_ctx_stream(None) is None
    assert lib.gops_ctx_scores_device(None) is None
    assert lib.gops_warm_count(None, 0) == -1
    assert lib.gops_graph_info(None, None, None, None) == _native.GOPS_ERR_INVALID


def _no_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")


def test_no_silent_cpu_fallback_without_a_device():
    """Without a GPU every solve raises (no CPU code path); only the
    reference's n == 0 early return needs no device."""
    _no_device()
    g = go.CsrAdjacency(np.array([0, 1, 2, 3]), np.array([1, 2, 0], np.int32), np.ones(3))
    cfg = go.PageRankConfig()
    for call in (lambda: go.pagerank_run(g, cfg), lambda: go.pagerank_weighted_run(g, cfg),
                 lambda: go.personalized_pagerank_run(g, cfg, [1.0, 0.0, 0.0]),
                 lambda: go.katz_centrality_run(g, go.KatzConfig()),
                 lambda: go.eigenvector_centrality_run(g, 100, 1e-6)):
        with pytest.raises(go.GopsError) as ei:
            call()
        assert ei.value.code == _native.GOPS_ERR_NO_DEVICE
    empty = go.pagerank_run(go.CsrAdjacency(np.array([0]), np.array([], np.int32)), cfg)
    assert empty.scores.size == 0 and empty.iterations == 0 and empty.converged


def test_bench_gpu_arm_fails_without_a_device():
    """bench.py's own arm has no CPU path either: no JSON line, non-zero exit."""
    _no_device()
    import subprocess
    import sys
    from conftest import ROOT
    r = subprocess.run([sys.executable, "bench.py", "--steps", "1", "--warmup", "3", "--scale", "10", "--no-cpu"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode != 0 and not any(x.startswith("{") for x in r.stdout.splitlines())


STRUCTS = [("gops_config", "Config"), ("gops_run", "Run"), ("gops_stats", "Stats"),
           ("gops_katz_config", "KatzConfig"), ("gops_warm_config", "WarmConfig"),
           ("gops_warm_stats", "WarmStats")]


def test_ctypes_structs_match_the_header(tmp_path):
    """Every struct the Python binding passes through the ABI has the C
    header's size, field names, field offsets and field sizes (compiled with
    the host C compiler against include/gops.h)."""
    import shutil
    import subprocess
    from conftest import ROOT
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gops.h"', 'int main(void) {']
    for cname, pyname in STRUCTS:
        lines.append(f'  printf("{pyname} size %zu\\n", sizeof({cname}));')
        for fname, _ in getattr(_native, pyname)._fields_:
            lines.append(f'  printf("{pyname} {fname} %zu %zu\\n", offsetof({cname}, {fname}), '
                         f'sizeof((({cname} *)0)->{fname}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", f"{ROOT}/include", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            parts = ln.split()
            got[tuple(parts[:2])] = tuple(int(x) for x in parts[2:])
    for _, pyname in STRUCTS:
        cls = getattr(_native, pyname)
        assert got[(pyname, "size")] == (ctypes.sizeof(cls),), pyname
        for fname, ftype in cls._fields_:
            desc = getattr(cls, fname)
            assert got[(pyname, fname)] == (desc.offset, ctypes.sizeof(ftype)), (pyname, fname)


SCALARS = {"int": ctypes.c_int, "int32_t": ctypes.c_int32, "int64_t": ctypes.c_int64, "uint64_t": ctypes.c_uint64,
           "size_t": ctypes.c_size_t, "double": ctypes.c_double, "float": ctypes.c_float}


def header_prototypes():
    import re
    from conftest import ROOT
    src = open(f"{ROOT}/include/gops.h").read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(gops_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        params = [p.strip() for p in m.group(3).split(",") if p.strip() and p.strip() != "void"]
        protos[m.group(2)] = (m.group(1).strip(), params)
    return protos


def test_ctypes_signatures_match_the_header():
    """Arity, and for each parameter pointer-or-scalar (scalars of the same C
    type), of every binding signature against include/gops.h's prototypes;
    the return kinds likewise."""
    protos = header_prototypes()
    for name, res, args in _native.SIGNATURES:
        ret, params = protos[name]
        assert len(params) == len(args), name
        for p, a in zip(params, args):
            if "*" in p:
                assert a in (ctypes.c_void_p, ctypes.c_char_p) or issubclass(a, ctypes._Pointer), (name, p)
            else:
                ctype = " ".join(w for w in p.replace("const ", "").split()[:-1])
                assert SCALARS[ctype] is a or ctypes.sizeof(SCALARS[ctype]) == ctypes.sizeof(a) and \
                    (SCALARS[ctype] in (ctypes.c_double, ctypes.c_float)) == (a in (ctypes.c_double, ctypes.c_float)), \
                    (name, p)
        if ret == "void":
            assert res is None, name
        elif "*" in ret:
            assert res in (ctypes.c_void_p, ctypes.c_char_p), name
        else:
            assert res is SCALARS[ret.replace("const ", "").strip()] or \
                ctypes.sizeof(res) == ctypes.sizeof(SCALARS[ret.strip()]), name


def test_score_buffer_arguments():
    """The batched calls' destination: True a new (nsets, n) float32 array,
    False none, a caller's array used as it is when it is C-contiguous float32
    of that shape, and anything else refused before the library is called."""
    a = _native.score_buffer(True, 3, 5)
    assert a.shape == (3, 5) and a.dtype == np.float32
    assert _native.score_buffer(False, 3, 5) is None
    mine = np.empty((3, 5), np.float32)
    assert _native.score_buffer(mine, 3, 5) is mine
    for bad in (np.empty((3, 5), np.float64), np.empty((2, 5), np.float32),
                np.empty((5, 3), np.float32).T):
        with pytest.raises(ValueError, match="float32 array of shape"):
            _native.score_buffer(bad, 3, 5)
