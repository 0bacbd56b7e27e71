"""Build libmdgb.so in-tree for GB300 (sm_103a).

    python -m moldyn_gb300.build [--force]

Translation units are compiled in parallel with nvcc and linked into
``moldyn_gb300/_build/libmdgb.so``.  ``kernels_step.cu`` is compiled with
``-fmad=false`` so its FP64 integrator/reduction arithmetic keeps the
reference's unfused rounding; the force kernels rely on explicit
round-to-nearest intrinsics for their FP64 path and may fuse FP32 maths.
Host C++ is compiled with ``-ffp-contract=off`` and portable flags only (the
same sources build on x86_64 and aarch64).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmdgb.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-I", INCLUDE, "--expt-relaxed-constexpr"]

UNITS = [
    ("kernels_step.cu", ["-fmad=false"]),
    ("kernels_force.cu", []),
    ("kernels_list.cu", []),
    ("engine.cu", []),
    ("host_util.cpp", []),
    ("noalloc.cu", []),
    ("splat.cu", []),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _sources():
    return [os.path.join(CSRC, u) for u, _ in UNITS] + [
        os.path.join(CSRC, "mdgb_internal.cuh"), os.path.join(INCLUDE, "mdgb.h"), __file__]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    procs = []
    objs = []
    for unit, extra in UNITS:
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT_DIR, unit + ".o")
        objs.append(obj)
        if unit.endswith(".cpp"):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
                   "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
        else:
            cmd = [nvcc()] + NVCC_COMMON + extra + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((unit, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(f"--- {u} ---\n{o}" for u, o in failed)
        raise RuntimeError(f"libmdgb build failed:\n{msg}")
    tmp = LIB + ".tmp"
    link = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(link))
    subprocess.check_call(link)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
