"""The C++ host API (graphops.hpp) runs the reference's own tests."""
import os
import subprocess

import pytest

from conftest import ROOT

LIB = os.path.join(ROOT, "graphops_gb300", "libgops.so")


@pytest.mark.skipif(not os.path.exists(LIB), reason="libgops.so not built")
def test_cpp_api_validation_and_adapters():
    import cpp_build
    exe = cpp_build.build()
    r = subprocess.run([exe, "--cpu-only"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_api_reference_tests_on_gpu():
    import cpp_build
    exe = cpp_build.build()
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout
