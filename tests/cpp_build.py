"""Builds tests/cpp/test_graphops (the C++ host API test) against libgops.so."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpp", "test_graphops.cpp")
OUT = os.path.join(HERE, "cpp", "test_graphops")


def build():
    lib_dir = os.path.join(ROOT, "graphops_gb300")
    hdrs = [os.path.join(ROOT, "graphops_gb300", "cpp", "graphops.hpp"), os.path.join(ROOT, "include", "gops.h")]
    newest = max(os.path.getmtime(p) for p in [SRC, os.path.join(lib_dir, "libgops.so")] + hdrs)
    if os.path.exists(OUT) and os.path.getmtime(OUT) >= newest:
        return OUT
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-o", OUT, SRC,
                           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "graphops_gb300", "cpp"),
                           "-L", lib_dir, "-lgops", f"-Wl,-rpath,{lib_dir}"])
    return OUT
