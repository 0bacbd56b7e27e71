"""GPU parity of the coupled configurations and the engine's failure and
reuse paths, against the oracle (through the C ABI).

* The mixed path with Berendsen thermostat and barostat (the 8M-atom
  configuration's coupling, tau* 0.5 -> T* 0.72, barostat beta 1, tau_P* 5 ->
  P* 1.0), scaled down to 1,792 atoms, against the oracle's FP64 run of the
  same steps (integrator.rs:14-59, thermostat.rs:24-34, barostat.rs:21-49).
  Bars, from the mixed path's force error (~1e-6 of the rms force):
  temperature and pressure then differ by ~1e-7..1e-6 relative, so lambda =
  sqrt(1 + dt/tau (T0/T - 1)) and mu = cbrt(1 + dt beta/tau (P - P0)) differ
  by at most ~dt/tau * 1e-6 ~ 1e-8 (measured on a GB300: lambda 1.4e-10, mu
  7.4e-10), the box (scaled by mu every step) by up to ~40 x that (measured
  9e-10, bar 2e-8), positions by ~1e-7 (bar 1e-6; the mixed NVE bar is 1e-5).
* A persistent, mixed ensemble with CUDA graphs of uneven replicas, each with
  its own thermostat and barostat targets, one of them in brute mode (box
  under 5 sigma): every replica against its own oracle run, same bars.
* Momentum (mod.rs:28-34) against the oracle, and the reference's momentum
  property (solver/src/lib.rs:59-75: 8 argon atoms, |sum v| < 1e-12 after
  every step) through the engine for 10,000 steps.
* The step kernel's bounded grid barrier made to run out (one block held
  back, a short wait limit): MDGB_ERR_DEVICE_TIMEOUT, no device fault, and
  the engine continues from the state the failed call started from.
* Graph chunks of every length, graph capture ahead of the call, uploads of
  the same shape that keep allocations and graphs, partial downloads.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import gpu_systems as gs

pytestmark = pytest.mark.gpu

T_STAR, TAU_T, BETA, TAU_P, P_STAR, DT = 0.72, 0.5, 1.0, 5.0, 1.0, 0.005


@pytest.fixture(scope="module")
def Engine():
    from moldyn_gb300 import _lib
    from moldyn_gb300.engine import Engine as E
    _lib.load()
    return E


def _oracle(oracle, pos, vel, box, mass=1.0, sigma=1.0, eps=1.0):
    st = oracle.OracleState([len(pos)], pos, vel, [mass], np.asarray(box, dtype=np.float64),
                            oracle.pot_table(1, default=(sigma, eps)))
    st.update_force()
    return st


def _min_image(d, box):
    return d - box * np.round(d / box)


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


# --------------------------------------------------------------------------
# mixed path + Berendsen T and P

def test_mixed_berendsen_thermostat_and_barostat_vs_oracle(Engine, oracle):
    from moldyn_gb300.initializer import Barostat, Thermostat
    pos, vel, box = gs.fcc((8, 8, 7), jitter=0.03, seed=61, t_star=1.0)
    T0 = gs.t_ref(T_STAR)
    e = Engine(precision="mixed")
    e.set_potential(0, 0, 1.0, 1.0)
    e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], box)
    e.compute_forces()
    ost = _oracle(oracle, pos, vel, box)
    th, ba = Thermostat.Berendsen(TAU_T), Barostat.Berendsen(BETA, TAU_P)
    oth, oba = oracle.Thermostat(oracle.BERENDSEN, TAU_T, 0.0, 0.0), oracle.Barostat(BETA, TAU_P, 0.0)
    worst = {"lambda": 0.0, "myu": 0.0, "box": 0.0, "pos": 0.0}
    for chunk in (1, 9, 30):
        e.step(chunk, DT, thermostat=th, target_temperature=T0, barostat=ba, target_pressure=P_STAR)
        ost.step(DT, nsteps=chunk, barostat=oba, P0=P_STAR, thermostat=oth, T0=T0)
        out = e.download()
        worst["lambda"] = max(worst["lambda"], _rel(th.lambda_, oth.lambda_))
        worst["myu"] = max(worst["myu"], _rel(ba.myu, oba.myu))
        worst["box"] = max(worst["box"], float(np.max(np.abs(out["box"] / ost.box - 1.0))))
        worst["pos"] = max(worst["pos"], float(np.abs(_min_image(out["pos"] - ost.pos, ost.box)).max()))
    print("mixed Berendsen T+P vs oracle:", worst)
    assert oth.lambda_ != 1.0 and oba.myu != 1.0 and not np.array_equal(ost.box, box)   # coupling acted
    assert worst["lambda"] <= 1e-8 and worst["myu"] <= 1e-8, worst
    assert worst["box"] <= 2e-8 and worst["pos"] <= 1e-6, worst
    e.close()


def _ensemble_systems():
    """Uneven replicas: a brute-mode crystal (box 3.4 < 5 sigma), a sparse gas,
    a crystal with one axis under three list radii, a dilute crystal and a
    dense one."""
    return [gs.fcc((2, 2, 2), seed=71, t_star=1.3),
            gs.gas(90, (9.0, 9.0, 9.0), seed=72),
            gs.fcc((5, 4, 3), jitter=0.05, seed=73, t_star=0.9),
            gs.fcc((6, 6, 6), rho=0.6, jitter=0.04, seed=74, t_star=1.6),
            gs.fcc((7, 7, 7), jitter=0.03, seed=75, t_star=0.6)]


def test_persistent_mixed_ensemble_with_coupling_vs_oracle(Engine, oracle):
    from moldyn_gb300.initializer import Barostat, Thermostat
    systems = _ensemble_systems()
    assert systems[0][2].max() < 5.0
    offs = np.cumsum([0] + [len(s[0]) for s in systems])
    pos = np.concatenate([s[0] for s in systems])
    vel = np.concatenate([s[1] for s in systems])
    boxes = np.array([s[2] for s in systems])
    T0s = [gs.t_ref(t) for t in (1.0, 0.8, 0.7, 1.4, 0.72)]
    P0s = [0.5, 0.05, 1.5, 0.8, 1.0]
    e = Engine(precision="mixed", persistent=True, graph_steps=10)
    e.set_potential(0, 0, 1.0, 1.0)
    e.upload_ensemble(offs, np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], boxes)
    e.compute_forces()
    ths = [Thermostat.Berendsen(TAU_T) for _ in systems]
    bas = [Barostat.Berendsen(BETA, TAU_P) for _ in systems]
    e.ensemble_set_coupling(ths, T0s, bas, P0s)
    e.ensemble_step(30, DT)
    e.ensemble_get_coupling()
    out = e.download()
    st = e.stats()
    assert st.graph_launches > 0
    for r, (p, v, b) in enumerate(systems):
        ost = _oracle(oracle, p, v, b)
        oth, oba = oracle.Thermostat(oracle.BERENDSEN, TAU_T, 0.0, 0.0), oracle.Barostat(BETA, TAU_P, 0.0)
        ost.step(DT, nsteps=30, barostat=oba, P0=P0s[r], thermostat=oth, T0=T0s[r])
        sl = slice(offs[r], offs[r + 1])
        dpos = float(np.abs(_min_image(out["pos"][sl] - ost.pos, ost.box)).max())
        dl, dm = _rel(ths[r].lambda_, oth.lambda_), _rel(bas[r].myu, oba.myu)
        dbox = float(np.max(np.abs(out["box"][r] / ost.box - 1.0)))
        print(f"replica {r} ({len(p)} atoms): pos {dpos:.2e} lambda {dl:.2e} myu {dm:.2e} box {dbox:.2e}")
        assert dpos <= 1e-6 and dl <= 1e-8 and dm <= 2e-8 and dbox <= 2e-8, r
    e.close()


# --------------------------------------------------------------------------
# momentum

@pytest.mark.parametrize("precision,ref", [("fp64", True), ("fp64", False), ("mixed", False)])
def test_momentum_matches_oracle(Engine, oracle, precision, ref):
    """get_momentum_of_system (mod.rs:28-34): bit-identical in reference
    order, 1e-13 of sum m|v| otherwise."""
    pos, vel, box = gs.fcc((6, 6, 6), jitter=0.05, seed=81)
    vel = vel + np.array([0.25, -0.125, 0.5])
    e = Engine(precision=precision, reference_order=ref)
    e.set_potential(0, 0, 1.0, 1.0)
    e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [2.0], box)
    e.compute_forces()
    m = e.macro(0)
    ost = _oracle(oracle, pos, vel, box, mass=2.0)
    want = ost.momentum()
    if ref:
        assert np.array_equal(m["momentum"], want)
    else:
        assert np.abs(m["momentum"] - want).max() <= 1e-13 * 2.0 * np.abs(vel).sum()
    e.close()


@pytest.mark.parametrize("precision,ref", [("fp64", True), ("mixed", False)])
def test_momentum_property_10k_steps(Engine, precision, ref):
    """solver/src/lib.rs:59-75 through the engine: 8 argon atoms on a 2x2x2
    lattice (edge 3.338339 nm), Maxwell-Boltzmann at 273.15 K with the +/-
    pairing, NVE Verlet at dt 0.002; |sum v| < 1e-12 after every one of
    10,000 steps."""
    from tests import refcases as rc
    from moldyn_gb300.initializer import maxwell_boltzmann
    pos, box = rc.lattice_argon_8()
    vel = maxwell_boltzmann(8, 273.15, 66.335, seed=3)
    e = Engine(precision=precision, reference_order=ref)
    e.set_potential(0, 0, 0.3418, 1.712)
    e.upload(np.zeros(8, dtype=np.uint16), pos, vel, [66.335], box)
    e.compute_forces()
    buf = {}
    worst = 0.0
    for _ in range(10000):
        e.step(1, 0.002)
        p = e.download(buf, fields=("vel",))["vel"].sum(axis=0)
        worst = max(worst, float(np.abs(p).max()))
        assert np.all(np.abs(p) < 1e-12)
    print(f"{precision}: max |sum v| over 10,000 steps {worst:.2e}")
    e.close()


# --------------------------------------------------------------------------
# failure path: the bounded grid barrier

@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_grid_barrier_timeout_is_reported_and_engine_recovers(Engine, oracle, precision):
    from moldyn_gb300 import _lib
    pos, vel, box = gs.fcc((8, 8, 8), jitter=0.03, seed=91)
    ref = _oracle(oracle, pos, vel, box)
    clean = Engine(precision=precision, threads_per_atom=1)
    clean.set_potential(0, 0, 1.0, 1.0)
    clean.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], box)
    clean.compute_forces()
    clean.step(12, DT)
    want = clean.download()
    clean.close()
    e = Engine(precision=precision, threads_per_atom=1)
    e.set_potential(0, 0, 1.0, 1.0)
    e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], box)
    e.compute_forces()
    before = e.download()
    e.test_barrier_timeout(hold_block=3, wait_cycles=200_000)
    with pytest.raises(_lib.MdgbError) as ei:
        e.step(5, DT)
    assert ei.value.status == 7          # MDGB_ERR_DEVICE_TIMEOUT
    after = e.download()
    for k in ("pos", "vel", "force"):
        assert np.array_equal(after[k], before[k]), k
    e.step(12, DT)                        # the engine carries on from the same state
    got = e.download()
    for k in ("pos", "vel", "force"):
        assert np.array_equal(got[k], want[k]), k
    ref.step(DT, nsteps=12)
    assert np.abs(_min_image(got["pos"] - ref.pos, box)).max() <= 1e-5
    e.close()


# --------------------------------------------------------------------------
# graphs, uploads, downloads

def test_graph_every_chunk_length_matches_eager(Engine):
    """graph_steps 8 over 21 steps: chunks of 8, 8 and 5, all replayed as
    graphs (captured ahead by prepare_step), bit-identical to eager."""
    pos, vel, box = gs.fcc((8, 8, 8), jitter=0.04, seed=95)
    outs, st = [], []
    for kw in ({}, dict(graph_steps=8)):
        e = Engine(precision="mixed", threads_per_atom=2, **kw)
        e.set_potential(0, 0, 1.0, 1.0)
        e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], box)
        e.compute_forces()
        e.prepare_step(21, DT)
        e.reset_stats()
        e.step(21, DT)
        outs.append(e.download())
        st.append(e.stats())
        e.close()
    for k in ("pos", "vel", "force", "potential", "temp"):
        assert np.array_equal(outs[0][k], outs[1][k]), k
    assert st[0].graph_launches == 0 and st[1].graph_launches == 3


def test_upload_same_shape_reuses_and_matches_fresh_engine(Engine):
    """A second upload of the same shape keeps the engine's allocations and
    graphs; its results equal a fresh engine's on that state."""
    a = gs.fcc((8, 8, 8), jitter=0.04, seed=96)
    b = gs.fcc((8, 8, 8), jitter=0.05, seed=97, t_star=1.1)
    e = Engine(precision="mixed", graph_steps=10, threads_per_atom=2)
    e.set_potential(0, 0, 1.0, 1.0)
    for pos, vel, box in (a, b):
        e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], box)
        e.compute_forces()
        e.step(20, DT)
    got = e.download()
    e.close()
    f = Engine(precision="mixed", graph_steps=10, threads_per_atom=2)
    f.set_potential(0, 0, 1.0, 1.0)
    f.upload(np.zeros(len(b[0]), dtype=np.uint16), b[0], b[1], [1.0], b[2])
    f.compute_forces()
    f.step(20, DT)
    want = f.download()
    f.close()
    for k in ("pos", "vel", "force", "potential", "temp"):
        assert np.array_equal(got[k], want[k]), k


def test_partial_download_and_buffer_reuse(Engine):
    pos, vel, box = gs.fcc((6, 6, 6), jitter=0.04, seed=98)
    e = Engine(precision="mixed")
    e.set_potential(0, 0, 1.0, 1.0)
    e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], box)
    e.compute_forces()
    e.step(7, DT)
    full = e.download()
    buf = {"pos": np.full((len(pos), 3), np.nan)}
    part = e.download(buf, fields=("pos", "temp"))
    assert part is buf and np.array_equal(part["pos"], full["pos"]) and np.array_equal(part["temp"], full["temp"])
    assert "vel" not in part
    e.close()


def test_bad_type_id_is_rejected_and_engine_stays_usable(Engine):
    from moldyn_gb300 import _lib
    pos, vel, box = gs.fcc((4, 4, 4), jitter=0.02, seed=99)
    e = Engine(precision="mixed")
    e.set_potential(0, 0, 1.0, 1.0)
    types = np.zeros(len(pos), dtype=np.uint16)
    types[5] = 3
    with pytest.raises(_lib.MdgbError) as ei:
        e.upload(types, pos, vel, [1.0], box)
    assert ei.value.status == 1
    e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], box)
    e.compute_forces()
    e.step(3, DT)
    e.close()


# --------------------------------------------------------------------------
# Nose-Hoover with several particle types

@pytest.mark.parametrize("precision,ref,tol", [("fp64", True, 1e-10), ("fp64", False, 1e-10),
                                               ("mixed", False, 1e-6)])
def test_nose_hoover_two_types_vs_oracle(Engine, oracle, precision, ref, tol):
    """Two types with their own masses and LJ pairs under one Nose-Hoover
    thermostat: psi gains psi_dot(T_t) * dt/2 once per type before the kick
    and once per type after it (thermostat.rs:35-39, 59-65, called per type
    from integrator.rs:23-26, 35-39); every type is scaled by the lambda
    computed before the kick.  lambda = exp(.) uses CUDA's exp against the C
    library's (an ulp apart at most), so FP64 agrees to 1e-10 over 40 steps;
    the mixed path to its force error."""
    from moldyn_gb300.initializer import Thermostat
    pos, vel, box = gs.fcc((5, 5, 5), jitter=0.04, seed=101, t_star=1.2)
    n = len(pos)
    types = (np.arange(n) % 3 == 0).astype(np.uint16)
    order = np.argsort(types, kind="stable")          # the oracle wants type-major order
    pairs = {(0, 0): (1.0, 1.0), (0, 1): (1.1, 0.8), (1, 1): (0.9, 1.3)}
    masses = [1.0, 2.0]
    ost = oracle.OracleState([int((types == 0).sum()), int((types == 1).sum())], pos[order], vel[order],
                             masses, box, oracle.pot_table(2, pairs))
    ost.update_force()
    e = Engine(precision=precision, reference_order=ref)
    for (a, b), (s, ep) in pairs.items():
        e.set_potential(a, b, s, ep)
    e.upload(types, pos, vel, masses, box)
    e.compute_forces()
    th = Thermostat.NoseHoover(0.4)
    oth = oracle.Thermostat(oracle.NOSE_HOOVER, 0.4, 0.0, 0.0)
    T0 = gs.t_ref(0.72)
    for chunk in (1, 39):
        e.step(chunk, DT, thermostat=th, target_temperature=T0)
        ost.step(DT, nsteps=chunk, thermostat=oth, T0=T0)
        out = e.download()
        dpos = float(np.abs(_min_image(out["pos"][order] - ost.pos, box)).max())
        dvel = float(np.abs(out["vel"][order] - ost.vel).max())
        print(f"{precision} ref={ref}: psi {th.psi:.6e} vs {oth.psi:.6e}, pos {dpos:.2e}, vel {dvel:.2e}")
        assert abs(th.psi - oth.psi) <= tol * max(1.0, abs(oth.psi))
        assert abs(th.lambda_ - oth.lambda_) <= tol
        assert dpos <= tol and dvel <= tol * 10
    assert oth.psi != 0.0
    e.close()


# --------------------------------------------------------------------------
# skin tuning

def test_skin_tuning_leaves_no_trace(Engine):
    """skin < 0: the first step call times a short stretch of steps with each
    candidate skin (0.08 .. 0.16 of r_cut) and puts the state back.  The run
    then equals, bit for bit, engines configured with the chosen skins (the
    same cell grids and lists) that start from the same forces -- those the
    tuned engine's compute_forces left, which the first kick uses -- on an
    ensemble with two size classes, replica by replica."""
    systems = [gs.fcc((5, 5, 5), jitter=0.04, seed=111), gs.fcc((9, 9, 9), jitter=0.04, seed=112)]
    offs = np.cumsum([0] + [len(s[0]) for s in systems])
    pos = np.concatenate([s[0] for s in systems])
    vel = np.concatenate([s[1] for s in systems])
    boxes = np.array([s[2] for s in systems])
    types = np.zeros(len(pos), dtype=np.uint16)
    a = Engine(precision="mixed", threads_per_atom=1, skin=-1.0)
    a.set_potential(0, 0, 1.0, 1.0)
    a.upload_ensemble(offs, types, pos, vel, [1.0], boxes)
    a.compute_forces()
    f0 = a.download()
    a.ensemble_step(30, DT)
    got = a.download()
    st = a.stats()
    a.close()
    cands = [f * 2.5 for f in (0.08, 0.10, 0.12, 0.14, 0.16)]
    present = [c for c in range(3) if st.class_replicas[c]]
    assert present == [0, 1]
    for c in present:
        assert min(abs(st.class_skin[c] - x) for x in cands) < 1e-12, st.class_skin
    print("tuned skins:", st.class_skin)
    for r, (p, v, bx) in enumerate(systems):
        sl = slice(offs[r], offs[r + 1])
        f = Engine(precision="mixed", threads_per_atom=1, skin=st.class_skin[r])
        f.set_potential(0, 0, 1.0, 1.0)
        f.upload(np.zeros(len(p), dtype=np.uint16), p, v, [1.0], bx)
        f.upload_forces(f0["force"][sl], f0["potential"][sl], f0["temp"][sl])
        f.step(30, DT)
        w = f.download()
        f.close()
        for k in ("pos", "vel", "force"):
            assert np.array_equal(got[k][sl], w[k]), (r, k)


def test_macro_getters_share_one_reduction(Engine):
    """The reference's getters (one per quantity, mod.rs / energy.rs /
    pressure.rs) read one cached reduction until the state changes."""
    from moldyn_gb300 import macro_parameters as mp
    from moldyn_gb300.core import ParticleDatabase, State
    from moldyn_gb300.solver import PotentialsDatabase, set_precision, update_force
    set_precision("mixed")
    ParticleDatabase.add(0, "test_particle", 1.0, 0.1)
    pos, vel, box = gs.fcc((4, 4, 4), jitter=0.03, seed=121)
    st = State(pos, vel, [0] * len(pos), box)
    update_force(PotentialsDatabase(), st)
    eng = st._engine
    n0 = eng.stats().kernel_launches
    vals = [mp.get_kinetic_energy(st, 0), mp.get_thermal_energy(st, 0), mp.get_potential_energy(st, 0),
            mp.get_pressure(st, 0), mp.get_center_of_mass_velocity(st, 0), mp.get_momentum_of_system(st, 0)]
    assert eng.stats().kernel_launches - n0 == 1
    m = eng.macro(0)
    assert vals[0] == m["kinetic_energy"] and vals[3] == m["pressure"]
    eng.step(1, DT)
    assert mp.get_kinetic_energy(st, 0) == eng.macro(0)["kinetic_energy"]
    set_precision("fp64")


# --------------------------------------------------------------------------
# exact sums of the coupled reductions (mixed path, from 65,536 atoms)

@pytest.mark.parametrize("layout", ["single", "ensemble"])
def test_exact_coupled_sums_match_the_fp64_reductions(Engine, layout):
    """From 65,536 atoms the mixed path's coupled step sums velocities, |v|^2,
    temp and potential exactly in 128-bit fixed point.  Its first step's
    lambda and mu must equal the Berendsen formulas (thermostat.rs:31-34,
    barostat.rs:29-30) evaluated on the temperature and pressure of the FP64
    macro-parameter reduction of the same state, to 1e-14 (the two sums
    differ by FP64 rounding only; cbrt/sqrt are CUDA's against numpy's)."""
    from moldyn_gb300.initializer import Barostat, Thermostat
    if layout == "single":
        systems = [gs.fcc((26, 26, 26), jitter=0.03, seed=131, t_star=1.1)]           # 70,304 atoms
    else:
        systems = [gs.fcc((20, 20, 20), jitter=0.03, seed=132, t_star=0.9),           # 32,000
                   gs.fcc((16, 16, 20), jitter=0.03, seed=133, t_star=1.4),           # 20,480
                   gs.fcc((15, 15, 15), rho=0.7, jitter=0.03, seed=134, t_star=1.2)]  # 13,500
        systems.append(gs.fcc((6, 6, 6), jitter=0.03, seed=135, t_star=0.8))          # 864
    offs = np.cumsum([0] + [len(s[0]) for s in systems])
    assert offs[-1] >= 65536
    pos = np.concatenate([s[0] for s in systems])
    vel = np.concatenate([s[1] for s in systems]) + 0.01 * np.arange(len(offs) - 1).repeat(np.diff(offs))[:, None]
    boxes = np.array([s[2] for s in systems])
    e = Engine(precision="mixed")
    e.set_potential(0, 0, 1.0, 1.0)
    types = np.zeros(len(pos), dtype=np.uint16)
    if layout == "single":
        e.upload(types, pos, vel, [1.0], boxes[0])
    else:
        e.upload_ensemble(offs, types, pos, vel, [1.0], boxes)
    e.compute_forces()
    mac = e.macro(0)
    macs = [mac] if layout == "single" else mac
    T0s = [gs.t_ref(0.72 + 0.1 * r) for r in range(len(systems))]
    P0s = [1.0 - 0.2 * r for r in range(len(systems))]
    ths = [Thermostat.Berendsen(TAU_T) for _ in systems]
    bas = [Barostat.Berendsen(BETA, TAU_P) for _ in systems]
    if layout == "single":
        e.step(1, DT, thermostat=ths[0], target_temperature=T0s[0], barostat=bas[0], target_pressure=P0s[0])
    else:
        e.ensemble_set_coupling(ths, T0s, bas, P0s)
        e.ensemble_step(1, DT)
        e.ensemble_get_coupling()
    for r, m in enumerate(macs):
        lam = np.sqrt(1.0 + DT / TAU_T * (T0s[r] / m["temperature"] - 1.0))
        myu = np.cbrt(1.0 + DT * BETA / TAU_P * (m["pressure"] - P0s[r]))
        assert abs(ths[r].lambda_ - lam) <= 1e-14, (r, ths[r].lambda_, lam)
        assert abs(bas[r].myu - myu) <= 1e-14, (r, bas[r].myu, myu)
    e.close()
