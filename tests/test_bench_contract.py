"""bench.py on the CPU: the reference arm's JSON line (it times the oracle
port on the host cores, no GPU) and the roofline bookkeeping helpers."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "atom-steps/s" and d["value"] > 0
    assert d["config"]["workload"] == "lj_fcc_1M_nve" and d["config"]["atoms"] == 1_000_000
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_fused_fraction_and_roofline_bytes():
    sys.path.insert(0, ROOT)
    import bench
    # a chunk of n NVE steps fuses (n - 1) rounded down to even of its force passes
    assert bench.fused_fraction(1) == 0.0
    assert bench.fused_fraction(3) == pytest.approx(2 / 3)
    assert bench.fused_fraction(64) == pytest.approx(62 / 64)
    assert bench.fused_fraction(1000) == pytest.approx((15 * 62 + 38) / 1000)
    # list 4 B x 77.6 candidates + mirror, count, force, potential/temp, velocity
    assert bench.LIST_CANDIDATES == pytest.approx(77.6, abs=0.05)
    assert bench.BYTES_PER_ATOM_FORCE == pytest.approx(4 * bench.LIST_CANDIDATES + 108)
    # a fused pass adds the drift's state traffic and skips force + potential/temp stores
    assert bench.BYTES_PER_ATOM_DRIFT - bench.BYTES_PER_ATOM_FUSED_SKIP == 60
    t = bench.ncu_traffic_per_atom()
    assert t is None or 300.0 < t < 600.0


def test_headline_system_is_the_documented_workload():
    """1,000,000 atoms on FCC 50 x 50 x 100 cells at rho* 0.8442 (a = (4/rho*)^(1/3)),
    inside the box, seeded Maxwell-Boltzmann velocities with zero momentum at T* 0.72."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    pos, vel, box = bench.make_system(seed=1234)
    a = (4.0 / 0.8442) ** (1.0 / 3.0)
    assert pos.shape == (1_000_000, 3) and vel.shape == (1_000_000, 3)
    assert np.allclose(box, np.array([50, 50, 100]) * a)
    assert (pos >= 0).all() and (pos < box).all()
    assert len(pos) / np.prod(box) == pytest.approx(0.8442, rel=1e-12)
    assert np.abs(vel.sum(axis=0)).max() < 1e-6
    # reduced temperature from the kinetic energy (m = 1, 3N - 3 degrees of freedom ~ 3N)
    t_star = (vel ** 2).sum() / (3 * len(vel))
    assert t_star == pytest.approx(0.72, rel=0.01)
    pos2, vel2, _ = bench.make_system(seed=1234)
    assert np.array_equal(pos, pos2) and np.array_equal(vel, vel2)


def test_reference_arm_loads_no_product_code():
    """The reference arm builds its system with the oracle and times the
    oracle: the product package (and libmdgb.so) is never imported."""
    code = ("import sys, argparse; sys.path.insert(0, %r); import bench; "
            "bench.run_reference(argparse.Namespace(steps=1, warmup=3, gpus=1)); "
            "bad = [m for m in sys.modules if m.startswith('moldyn_gb300')]; "
            "assert not bad, bad" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][0])
    # the timed region is what ran: the sampled step's own time
    assert d["ms_per_step"] == pytest.approx(d["sampled_step"]["ms"])
    assert d["sampled_step"]["full_step_ms_extrapolated"] > d["ms_per_step"]


def test_reference_arm_positions_are_the_headline_system():
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    pos, vel, box = bench.make_system(seed=1234)
    opos, obox = bench.make_positions_oracle()
    assert np.array_equal(pos, opos) and np.array_equal(box, obox)
