"""CPU-side checks of libmdgb.so: it loads without a GPU, exports every symbol
include/mdgb.h declares, and its host-only helpers agree with the oracle."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

from tests import refcases as rc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "mdgb.h")).read()
    return sorted(set(re.findall(r"MDGB_API\s+[^;(]*?\b(mdgb_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from moldyn_gb300 import _lib
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    from moldyn_gb300 import _lib
    names = _declared()
    assert len(names) >= 29
    for name in names:
        assert hasattr(lib, name), f"{name} declared in include/mdgb.h but not exported"
    # the ctypes binding covers exactly the declared ABI
    assert sorted(_lib.SIGNATURES) == names


def test_abi_version(lib):
    assert lib.mdgb_abi_version() == 1


def test_lj_matches_golden_and_oracle(lib, oracle):
    """solver/src/lib.rs:77-89 through the C ABI's host helper."""
    out = np.zeros(4)
    assert lib.mdgb_lj_new(0.3418, 1.712, out) == 0
    assert np.array_equal(out, oracle.lj_new(0.3418, 1.712))
    u, f = C.c_double(), C.c_double()
    lib.mdgb_lj_eval(out, 0.5, C.byref(u), C.byref(f))
    want = {a["expr"]: a["value"] for a in rc.kats()["lennard_jones"]["asserts"]}
    assert rc.fmt8(u.value) == want["potential"] and rc.fmt8(f.value) == want["force"]
    for r in (0.3, 0.34, 0.41, 0.85, 0.8545, 0.9):
        lib.mdgb_lj_eval(out, r, C.byref(u), C.byref(f))
        assert (u.value, f.value) == oracle.lj_eval(out, r)


@pytest.mark.parametrize("kind,grid", [("U", (10, 10, 10)), ("FCC", (3, 4, 5))])
def test_lattice_matches_oracle(lib, oracle, kind, grid):
    from moldyn_gb300.initializer import UnitCell, lattice_positions
    got = lattice_positions(UnitCell[kind], grid, 1.6796, (0.1, 0.2, 0.3))
    want = oracle.lattice(kind, *grid, 1.6796, (0.1, 0.2, 0.3))
    assert np.array_equal(got, want)


def test_maxwell_boltzmann_properties(lib):
    from moldyn_gb300.initializer import maxwell_boltzmann
    v = maxwell_boltzmann(20001, 273.15, 66.335, seed=7)
    assert np.all(v[-1] == 0.0)                          # odd n: last atom keeps v = 0
    assert np.all(np.abs(v.sum(axis=0)) < 1e-12)         # +v / -v pairing
    sigma = np.sqrt(1.380648528 * 273.15 * 0.01 / 66.335)
    assert abs(v[:-1].std() / sigma - 1.0) < 0.02
    v2 = maxwell_boltzmann(20001, 273.15, 66.335, seed=7)
    assert np.array_equal(v, v2)                          # seeded and deterministic
    v3 = maxwell_boltzmann(20001, 273.15, 66.335, seed=8)
    assert not np.array_equal(v, v3)


def test_maxwell_boltzmann_golden_bits(lib):
    """The portable generator gives the same bits on every IEEE host."""
    from moldyn_gb300.initializer import maxwell_boltzmann
    v = maxwell_boltzmann(6, 100.0, 1.0, seed=12345)
    h = v[:3].tobytes().hex()
    golden = os.path.join(ROOT, "tests", "golden", "mb_seed12345.txt")
    assert open(golden).read().strip() == h


def test_create_without_gpu_fails_loudly(lib):
    """No silent CPU path: without a usable GPU, creating an engine errors."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from moldyn_gb300 import _lib
    from moldyn_gb300.engine import Engine
    with pytest.raises(_lib.MdgbError):
        Engine()


def test_status_strings(lib):
    for s in range(10):
        assert lib.mdgb_status_string(s)


def test_splat_rejects_bad_arguments_without_touching_a_gpu(lib):
    """mdgb_splat validates its arguments before any CUDA call: a camera that
    is not a symmetric perspective, an empty image or a missing buffer come
    back as MDGB_ERR_INVALID_ARGUMENT (1), here with no GPU at all."""
    from moldyn_gb300 import _lib
    from moldyn_gb300.render import Camera, splat_params
    parts = np.zeros((2, 12), dtype=np.float32)
    out = np.zeros((4, 4, 4), dtype=np.float32)
    prm = splat_params(Camera((0.0, 0.0, 0.0), 70.0, 4, 4))
    assert lib.mdgb_splat(parts, 2, C.byref(prm), 0, 4, out) == 1
    assert lib.mdgb_splat(parts, -1, C.byref(prm), 4, 4, out) == 1
    bad = _lib.CSplatParams()
    C.memmove(C.byref(bad), C.byref(prm), C.sizeof(prm))
    bad.proj[11] = 0.0          # not a perspective projection
    assert lib.mdgb_splat(parts, 2, C.byref(bad), 4, 4, out) == 1


def test_trace_flag_and_phase_names():
    """MDGB_FLAG_TRACE and the phase names mdgb_trace_phases reports."""
    from moldyn_gb300 import _lib
    assert _lib.FLAG_TRACE == 8
    assert len(_lib.TRACE_PHASES) == 14 and _lib.TRACE_PHASES[-2:] == ["launches", "rebuild_launches"]
    src = open(os.path.join(ROOT, "include", "mdgb.h")).read()
    assert "#define MDGB_FLAG_TRACE 8u" in src


def test_noalloc_validates_arguments_on_the_host(lib):
    """mdgb_forces_noalloc rejects a box that is not positive and finite, and
    a non-finite sigma, before any CUDA call (no device pointer is touched)."""
    for box in ([np.inf, 10.0, 10.0], [10.0, np.nan, 10.0], [10.0, 10.0, -1.0], [0.0, 10.0, 10.0]):
        assert lib.mdgb_forces_noalloc(10, 1, np.array(box), 1.0, 1.0, 1, None, None, None) == 1
    assert lib.mdgb_forces_noalloc(10, 1, np.array([10.0, 10.0, 10.0]), np.nan, 1.0, 1, None, None, None) == 1
    assert lib.mdgb_forces_noalloc(10, 1, np.array([10.0, 10.0, 10.0]), 1.0, np.inf, 1, None, None, None) == 1


def test_noalloc_huge_box_grid_terminates_without_a_gpu(lib):
    """A box of 1e12 passes validation; the cell grid is coarsened in closed
    form (no per-cell loop), and without a GPU the call ends with a CUDA error
    instead of launching anything."""
    import time

    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the GPU test covers this box with real buffers)")
    t0 = time.perf_counter()
    st = lib.mdgb_forces_noalloc(10, 1, np.array([1e12, 1e12, 1e12]), 1.0, 1.0, 1, None, None, None)
    assert st == 2 and time.perf_counter() - t0 < 5.0
