"""Build recipe for the oracle's C restatement (test infrastructure).

Compiles ``oracle/pagerank_port.c`` into ``oracle/liborcport.so`` with gcc.
``-ffp-contract=off`` keeps FP64 results bit-identical between x86-64 and
AArch64 (no fused multiply-add contraction).

There is no ``oracle/_ref``: the reference is a Rust crate and no Rust
toolchain exists on either machine, so only this restatement is built.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "pagerank_port.c")
OUT = os.path.join(HERE, "liborcport.so")


def build(force: bool = False) -> str:
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= os.path.getmtime(SRC)):
        return OUT
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           "-std=c11", "-Wall", "-o", OUT, SRC, "-lm"]
    subprocess.check_call(cmd)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
