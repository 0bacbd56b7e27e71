"""mdgb_forces_noalloc: the allocation-free force entry point.

It serves callers that cannot allocate GPU memory (a plugin whose host
application owns every device allocation, a loop in which an allocation's
implicit device synchronisation is not allowed, a fixed memory budget).  The
caller brings device buffers for positions and results; the call's own
scratch is a static device array inside the library.

Checked here through the C ABI: calls in a row on different systems (a
27-cell liquid, a small single-cell gas, a slab one cell thick near the atom
limit, a huge sparse box) each agree with the oracle's update_force within
1e-12 of the force scale (per-pair arithmetic is the reference's; only the
summation order differs), and with the engine's FP64 entry point
(mdgb_compute_forces) to the same bar.  An over-size request is refused with
MDGB_ERR_NOALLOC_TOO_LARGE.  Device buffers for the test come from torch; the
entry point itself allocates nothing.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import gpu_systems as gs

pytestmark = pytest.mark.gpu


def _engine_forces(pos, box):
    from moldyn_gb300.engine import Engine
    e = Engine(precision="fp64")
    e.set_potential(0, 0, 1.0, 1.0)
    e.upload(np.zeros(len(pos), dtype=np.uint16), pos, np.zeros_like(pos), [1.0], box)
    e.compute_forces()
    out = e.download()
    e.close()
    return out


def _oracle_forces(oracle, pos, box):
    st = oracle.OracleState([len(pos)], pos, np.zeros_like(pos), [1.0], np.asarray(box, dtype=np.float64),
                            oracle.pot_table(1, default=(1.0, 1.0)))
    st.update_force()
    return st.force.copy(), st.potential.copy(), st.temp.copy()


def _noalloc_forces(lib, torch, pos, box):
    dev = torch.device("cuda:0")
    d_pos = torch.tensor(pos.reshape(-1), dtype=torch.float64, device=dev)
    d_f = torch.full((3 * len(pos),), float("nan"), dtype=torch.float64, device=dev)
    d_p = torch.full((len(pos),), float("nan"), dtype=torch.float64, device=dev)
    d_t = torch.full((len(pos),), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    st = lib.mdgb_forces_noalloc(len(pos), d_pos.data_ptr(), np.ascontiguousarray(box, dtype=np.float64),
                                 1.0, 1.0, d_f.data_ptr(), d_p.data_ptr(), d_t.data_ptr(), stream)
    assert st == 0, st
    torch.cuda.synchronize(dev)
    return d_f.cpu().numpy().reshape(-1, 3), d_p.cpu().numpy(), d_t.cpu().numpy()


def _close(got, want, tol=1e-12):
    scale = max(np.abs(want).max(), 1e-300)
    return np.abs(got - want).max() <= tol * scale


def _slab():
    """A slab thinner than three cut-off radii along z (one cell thick) with
    61,504 atoms: the other two axes keep their cell grid."""
    pos, vel, box = gs.fcc((62, 62, 4), rho=0.8442, jitter=0.03, seed=43)
    assert box[2] < 3 * 2.5 and len(pos) <= 65536
    return pos, box


def test_noalloc_matches_oracle_calls_in_a_row(oracle):
    torch = pytest.importorskip("torch")
    from moldyn_gb300 import _lib
    lib = _lib.load()
    systems = [gs.fcc((6, 6, 6), jitter=0.06, seed=41)[::2],          # 864 atoms, 27-cell stencil
               gs.gas(120, (7.0, 7.0, 7.0), seed=42)[::2]]            # small box: a single cell
    for _ in range(2):                                                # the array keeps the last call's contents
        for pos, box in systems:
            f, p, t = _noalloc_forces(lib, torch, pos, box)
            of, op, ot = _oracle_forces(oracle, pos, box)
            assert _close(f, of) and _close(p, op) and _close(t, ot)
            want = _engine_forces(pos, box)
            assert _close(f, want["force"]) and _close(p, want["potential"]) and _close(t, want["temp"])


def test_noalloc_slab_near_the_atom_limit(oracle):
    """One cell along the thin axis, a full stencil on the others; the rows of
    the oracle are sampled (all-pairs over 60k atoms)."""
    torch = pytest.importorskip("torch")
    from moldyn_gb300 import _lib
    lib = _lib.load()
    pos, box = _slab()
    f, p, t = _noalloc_forces(lib, torch, pos, box)
    st = oracle.OracleState([len(pos)], pos, np.zeros_like(pos), [1.0], box, oracle.pot_table(1, default=(1.0, 1.0)))
    rows = 4096
    st.update_force(rows=(0, rows))
    assert _close(f[:rows], st.force[:rows]) and _close(p[:rows], st.potential[:rows])
    assert _close(t[:rows], st.temp[:rows])


def test_noalloc_huge_sparse_box():
    """A box far larger than the cut-off: the grid is coarsened to the cell
    limit in closed form; isolated atoms feel no force."""
    torch = pytest.importorskip("torch")
    from moldyn_gb300 import _lib
    lib = _lib.load()
    box = np.array([1e12, 1e12, 1e12])
    pos = np.array([[1.0, 2.0, 3.0], [5e11, 5e11, 5e11], [9e11, 1e9, 3e10]])
    f, p, t = _noalloc_forces(lib, torch, pos, box)
    assert np.array_equal(f, np.zeros_like(f)) and np.array_equal(p, np.zeros(3))


def test_noalloc_rejects_oversize():
    from moldyn_gb300 import _lib
    lib = _lib.load()
    box = np.array([10.0, 10.0, 10.0])
    st = lib.mdgb_forces_noalloc(65537, 1, box, 1.0, 1.0, 1, None, None, None)
    assert st == 10   # MDGB_ERR_NOALLOC_TOO_LARGE
    # one cell on every axis (a box under three cut-off radii): at most 4096 atoms
    st = lib.mdgb_forces_noalloc(4097, 1, np.array([7.0, 7.0, 7.0]), 1.0, 1.0, 1, None, None, None)
    assert st == 10
