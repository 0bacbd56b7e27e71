"""Build recipe for the oracle (test infrastructure only).

Compiles ``oracle/mdref.cpp`` -- the CPU FP64 restatement of the moldyn
solver path -- into ``oracle/_build/libmdref.so``.  Portable flags only (the
same file builds on x86_64 and aarch64); ``-ffp-contract=off`` keeps every
``a*b + c`` as two rounded operations, as Rust evaluates it.

The reference itself is Rust and cannot be compiled here (no cargo/rustc), so
there is no ``oracle/_ref`` build; the restatement is pinned to the
reference's own golden test values instead.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mdref.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmdref.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", SRC, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
