"""Build recipes for the native parts of graphops_gb300.

* ``libgops.so``      the CUDA library behind include/gops.h (nvcc, sm_103a only)
* ``libgraphgen.so``  the seeded synthetic-graph generators (gcc)

Both land next to this file (in-tree, git-ignored).  Translation units are
compiled in parallel; a unit is rebuilt only when a source or header is newer
than its object file.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIBGOPS = os.path.join(PKG, "libgops.so")
LIBGEN = os.path.join(PKG, "libgraphgen.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_gops(force: bool = False, verbose: bool = False, extra: list | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    hdr_time = _newest(headers)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *(extra or []), "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or not os.path.exists(LIBGOPS) or os.path.getmtime(LIBGOPS) < _newest(objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIBGOPS, *objs, "-lcuda", "-lpthread"])
    return LIBGOPS


def build_graphgen(force: bool = False) -> str:
    src = os.path.join(PKG, "gen", "graphgen.c")
    hdr = os.path.join(PKG, "gen", "graphgen.h")
    if force or not os.path.exists(LIBGEN) or os.path.getmtime(LIBGEN) < _newest([src, hdr]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", "-std=c11",
              "-Wall", "-o", LIBGEN, src, "-lm"])
    return LIBGEN


def build_all(force: bool = False, verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_gops, force, verbose)
        f2 = ex.submit(build_graphgen, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIBGOPS)
