"""mdgb_forces_noalloc: the allocation-free force entry point.

It serves callers that cannot allocate GPU memory (a plugin whose host
application owns every device allocation, a loop in which an allocation's
implicit device synchronisation is not allowed, a fixed memory budget).  The
caller brings device buffers for positions and results; the call's own
scratch is a static device array inside the library.

Checked here through the C ABI: two calls in a row, on two different
systems, each agree with the engine's FP64 force entry point
(mdgb_compute_forces) within the FP64 tolerance the other parity tests use
(1e-12 of the largest force component), and an over-size request is refused
with MDGB_ERR_NOALLOC_TOO_LARGE.  Device buffers for the test come from torch;
the entry point itself allocates nothing.
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


def test_noalloc_matches_engine_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    from moldyn_gb300 import _lib
    lib = _lib.load()
    systems = [gs.fcc((6, 6, 6), jitter=0.06, seed=41),          # 864 atoms, 27-cell stencil
               gs.gas(120, (7.0, 7.0, 7.0), seed=42)]            # small box: a single cell
    for pos, _, box in systems:
        want = _engine_forces(pos, box)
        f, p, t = _noalloc_forces(lib, torch, pos, box)
        scale = np.abs(want["force"]).max()
        assert np.abs(f - want["force"]).max() <= 1e-12 * scale
        assert np.abs(p - want["potential"]).max() <= 1e-12 * np.abs(want["potential"]).max()
        assert np.abs(t - want["temp"]).max() <= 1e-12 * np.abs(want["temp"]).max()


def test_noalloc_rejects_oversize():
    from moldyn_gb300 import _lib
    lib = _lib.load()
    box = np.array([10.0, 10.0, 10.0])
    st = lib.mdgb_forces_noalloc(65537, 1, box, 1.0, 1.0, 1, None, None, None)
    assert st == 10   # MDGB_ERR_NOALLOC_TOO_LARGE
