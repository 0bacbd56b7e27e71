"""Host arithmetic of the engine, on the CPU: the r^2 threshold that replaces
the square root in the mixed path's exact pair test (host_math.h)."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sqrt_cut_matches_the_square_root_test(tmp_path):
    """sqrt_cut(rc) is the smallest double whose rounded square root exceeds
    rc, so r^2 < sqrt_cut(rc) decides exactly like sqrt(r^2) <= rc
    (potential.rs:201-204): 4000 cutoffs x 4000 doubles around each threshold."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "sqrt_cut_check")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                           os.path.join(ROOT, "tests", "cpp", "sqrt_cut_check.cpp"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "0 failures" in out.stdout
