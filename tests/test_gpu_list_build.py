"""The two Verlet-list builds (kernels_list.cu) give the same lists.

The paired build (replicas of at least 32,768 atoms) tests each pair of
neighbouring cells once and expands per-(atom, shift code) hit words; the
direct build (smaller replicas, MDGB_FLAG_DIRECT_LIST, and the engine's own
choice for a rebuild with a cell of more than 32 atoms) tests every cell
against its 27 neighbour cells.  Both list the same entries in the same
order, except a pair within rounding of rlist (1 + 1e-5) -- far outside
r_cut -- which the paired build decides once for both sides.  With one
thread per atom such an entry changes nothing (it is skipped), so every
result is compared with np.array_equal; with several threads per atom it
shifts the lanes' shares of the list, so the mixed path's forces (exact
fixed-point sums) and trajectory stay bit-identical while its FP32
potential/virial sums and the FP64 tree-order sums may move in the last
bits (tolerances below).  Which build ran is read from
mdgb_stats.direct_list_builds.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import gpu_systems as gs

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "force", "potential", "temp")
# FCC unit cells of a box whose cells (side >= 2.8 sigma) hold ~20 atoms
PAIRED_CELLS = (17, 17, 29)


@pytest.fixture(scope="module")
def Engine():
    from moldyn_gb300 import _lib
    from moldyn_gb300.engine import Engine
    _lib.load()
    return Engine


def _run(Engine, pos, vel, box, steps, types=None, ntypes=1, pots=((0, 0, 1.0, 1.0),), **kw):
    e = Engine(**kw)
    for t0, t1, s, eps in pots:
        e.set_potential(t0, t1, s, eps)
    ty = np.zeros(len(pos), dtype=np.uint16) if types is None else types
    e.upload(ty, pos, vel, [1.0] * ntypes, box)
    e.compute_forces()
    e.step(steps, 0.005)
    out = e.download()
    st = e.stats()
    e.close()
    return out, st


@pytest.mark.parametrize("precision,ref", [("mixed", False), ("fp64", True), ("fp64", False)])
def test_paired_build_equals_direct(Engine, precision, ref):
    # 33,524 atoms: 10 x 10 x 17 cells of ~20 atoms (the paired build's case)
    pos, vel, box = gs.fcc(PAIRED_CELLS, jitter=0.05, seed=41)
    kw = dict(precision=precision, reference_order=ref, threads_per_atom=1)
    a, sa = _run(Engine, pos, vel, box, 40, **kw)
    b, sb = _run(Engine, pos, vel, box, 40, direct_list=True, **kw)
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k
    assert sa.rebuilds >= 3 and sa.rebuilds == sb.rebuilds
    assert sa.direct_list_builds == 0
    assert sb.direct_list_builds >= sb.rebuilds


@pytest.mark.parametrize("precision,tpa", [("mixed", 4), ("fp64", 2)])
def test_paired_build_threads_per_atom(Engine, precision, tpa):
    pos, vel, box = gs.fcc(PAIRED_CELLS, jitter=0.05, seed=41)
    kw = dict(precision=precision, threads_per_atom=tpa)
    a, sa = _run(Engine, pos, vel, box, 40, **kw)
    b, sb = _run(Engine, pos, vel, box, 40, direct_list=True, **kw)
    if precision == "mixed":
        for k in ("pos", "vel", "force"):
            assert np.array_equal(a[k], b[k]), k
        for k in ("potential", "temp"):
            scale = np.sqrt(np.mean(b[k] ** 2))
            assert np.max(np.abs(a[k] - b[k])) <= 1e-6 * scale, k
    else:
        assert np.max(np.abs(a["pos"] - b["pos"])) <= 1e-10
        fs = np.max(np.abs(b["force"]))
        assert np.max(np.abs(a["force"] - b["force"])) <= 1e-9 * fs
    assert sa.direct_list_builds == 0 and sb.direct_list_builds > 0


def test_paired_build_multitype_equals_direct(Engine):
    """Two types with the reference's one-sided pairs (type t sees types >= t,
    potential.rs:171-176): the paired build decides each side by its own type."""
    pos, vel, box = gs.fcc(PAIRED_CELLS, jitter=0.05, seed=42)
    rng = np.random.default_rng(7)
    types = rng.integers(0, 2, len(pos)).astype(np.uint16)
    pots = ((0, 0, 1.0, 1.0), (0, 1, 0.95, 0.9), (1, 0, 0.95, 0.9), (1, 1, 0.9, 0.8))
    for precision, ref in (("mixed", False), ("fp64", True)):
        kw = dict(precision=precision, reference_order=ref, threads_per_atom=1)
        a, sa = _run(Engine, pos, vel, box, 30, types=types, ntypes=2, pots=pots, **kw)
        b, sb = _run(Engine, pos, vel, box, 30, types=types, ntypes=2, pots=pots, direct_list=True, **kw)
        for k in FIELDS:
            assert np.array_equal(a[k], b[k]), (precision, k)
        assert sa.direct_list_builds == 0 and sb.direct_list_builds > 0


def test_crowded_cells_take_the_direct_build(Engine):
    """A skin of 1 sigma makes cells of ~40 atoms: the engine falls back to the
    direct build by itself, with the same results as when asked for it."""
    pos, vel, box = gs.fcc(PAIRED_CELLS, jitter=0.05, seed=43)
    a, sa = _run(Engine, pos, vel, box, 20, precision="mixed", skin=1.0, threads_per_atom=1)
    b, sb = _run(Engine, pos, vel, box, 20, precision="mixed", skin=1.0, threads_per_atom=1, direct_list=True)
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k
    assert sa.direct_list_builds > 0


def test_paired_build_ensemble_equals_direct(Engine):
    """Replicas of uneven size (one in brute mode, small ones on the direct
    build, one on the paired build), persistent force kernel and graphs: both
    builds give the same trajectories."""
    systems = [gs.fcc((2, 2, 2), seed=44), gs.fcc((6, 5, 7), jitter=0.05, seed=45),
               gs.gas(300, (14.0, 14.0, 14.0), seed=46), gs.fcc((8, 8, 8), rho=0.7, seed=47),
               gs.fcc(PAIRED_CELLS, jitter=0.05, seed=48)]
    offs = np.cumsum([0] + [len(s[0]) for s in systems])
    pos = np.concatenate([s[0] for s in systems])
    vel = np.concatenate([s[1] for s in systems])
    boxes = np.array([s[2] for s in systems])
    outs, stats = [], []
    for direct in (False, True):
        e = Engine(precision="mixed", persistent=True, graph_steps=10, threads_per_atom=1, direct_list=direct)
        e.set_potential(0, 0, 1.0, 1.0)
        e.upload_ensemble(offs, np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], boxes)
        e.compute_forces()
        e.ensemble_step(30, 0.005)
        outs.append(e.download())
        stats.append(e.stats())
        e.close()
    for k in FIELDS:
        assert np.array_equal(outs[0][k], outs[1][k]), k
    assert stats[0].direct_list_builds == 0 and stats[1].direct_list_builds > 0
