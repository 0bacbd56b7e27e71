"""GPU parity: libmdgb (through the C ABI) against the oracle.

Tolerances (written per test):
  FP64 plain path, reference order   bit-identical forces/potential/temp and
                                     NVE / Berendsen-thermostat trajectories
  FP64 plain path, tree order        |dF| <= 1e-12 * max|F| per component
  mixed path                         max_i |dF_i| / max(|F_i|, rms|F|) <= 1e-5
                                     and rms|dF| / rms|F| <= 3e-6
  pair sets                          exactly equal to the all-pairs set
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import gpu_systems as gs
from tests import refcases as rc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mdgb():
    from moldyn_gb300 import _lib
    from moldyn_gb300.engine import Engine
    _lib.load()
    return Engine


def _engine(Engine, precision="fp64", ref=False, table=None, **kw):
    e = Engine(precision=precision, reference_order=ref, **kw)
    return e


def _oracle_state(oracle, pos, vel, box, mass=1.0, sigma=1.0, eps=1.0):
    n = len(pos)
    return oracle.OracleState([n], pos, vel, [mass], box, oracle.pot_table(1, default=(sigma, eps)))


def _upload(e, pos, vel, box, mass=1.0, sigma=1.0, eps=1.0):
    e.set_potential(0, 0, sigma, eps)
    e.upload(np.zeros(len(pos), dtype=np.uint16), pos, vel, [mass], box)


# --------------------------------------------------------------------------
# the reference's own known-answer tests, through the GPU

def test_kats_through_gpu_mirror_api(oracle):
    """solver/src/lib.rs:91-427 and cli/src/tests.rs:35-98 via the mirror API
    (FP64, reference order): golden strings and oracle bits."""
    from moldyn_gb300 import macro_parameters as mp
    from moldyn_gb300.core import ParticleDatabase, State
    from moldyn_gb300.solver import Integrator, PotentialsDatabase, set_precision, update_force
    set_precision("fp64")
    ParticleDatabase.add(0, "Argon", 66.335, 0.071)
    kats = rc.kats()
    counts, pos, vel, mass, box = rc.two_argon_moving()
    st = State(pos, vel, [0, 0], box)
    pdb = PotentialsDatabase()
    update_force(pdb, st)
    ost = oracle.OracleState(counts, pos, vel, mass, box, oracle.pot_table(1))
    ost.update_force()
    done = 0
    for name in ("verlet_with_lennard_jones", "verlet_lj_1000_iterations"):
        st = State(pos, vel, [0, 0], box)
        update_force(pdb, st)
        ost = oracle.OracleState(counts, pos, vel, mass, box, oracle.pot_table(1))
        ost.update_force()
        done = 0
        for a in sorted(kats[name]["asserts"], key=lambda r: r["after_steps"]):
            if a["after_steps"] > done:
                Integrator.VerletMethod.calculate(pdb, st, 0.002, steps=a["after_steps"] - done)
                ost.step(0.002, nsteps=a["after_steps"] - done)
                done = a["after_steps"]
            assert np.array_equal(st.positions, ost.pos) and np.array_equal(st.velocities, ost.vel)
            assert np.array_equal(st.forces, ost.force)
            q = {f"pos{k + 1}.{ax}": st.positions[k, i] for k in range(2) for i, ax in enumerate("xyz")}
            q.update({f"v{k + 1}.{ax}": st.velocities[k, i] for k in range(2) for i, ax in enumerate("xyz")})
            q.update({f"f{k + 1}.{ax}": st.forces[k, i] for k in range(2) for i, ax in enumerate("xyz")})
            if a["expr"] in q:
                assert rc.fmt8(q[a["expr"]]) == a["value"], a["source"]
    # 999-step macro parameters (solver/src/lib.rs:317-331)
    want = {a["expr"]: a["value"] for a in kats["verlet_lj_1000_iterations"]["asserts"]}
    ke = mp.get_kinetic_energy(st, 0)
    th = mp.get_thermal_energy(st, 0)
    pe = mp.get_potential_energy(st, 0)
    assert rc.fmt8(ke) == want["kinetic"] and rc.fmt8(th) == want["thermal"]
    assert rc.fmt8(pe) == want["potential"]
    assert rc.fmt8(mp.get_temperature(th, 2) / 100.0) == want["temperature / 100.0"]
    assert rc.fmt8(mp.get_pressure(st, 0)) == want["pressure"]


def test_energy_temperature_pressure_kats():
    """solver/src/lib.rs:334-427 through the GPU reductions."""
    from moldyn_gb300 import macro_parameters as mp
    from moldyn_gb300.core import ParticleDatabase, State
    from moldyn_gb300.solver import PotentialsDatabase, set_precision, update_force
    set_precision("fp64")
    ParticleDatabase.add(0, "Argon", 66.335, 0.071)
    kats = rc.kats()
    counts, pos, vel, mass, box = rc.two_argon_moving()
    st = State(pos, vel, [0, 0], box)
    update_force(PotentialsDatabase(), st)
    mv = mp.get_center_of_mass_velocity(st, 0)
    assert tuple(mv) == (0.0, 1.0, 0.0)
    ke, th, pe = mp.get_kinetic_energy(st, 0), mp.get_thermal_energy(st, 0), mp.get_potential_energy(st, 0)
    e = {a["expr"]: a["value"] for a in kats["energies"]["asserts"] if "value" in a}
    assert rc.fmt8(ke) == e["e_kinetic"] and rc.fmt8(th) == e["e_thermal"]
    assert rc.fmt8(pe) == e["e_potential"] and rc.fmt8(th + pe) == e["e_internal"]
    assert rc.fmt8(ke + pe) == e["e"]
    assert rc.fmt8(mp.get_temperature(th, 2)) == kats["temperature"]["asserts"][0]["value"]
    assert rc.fmt8(mp.get_pressure(st, 0)) == kats["pressure"]["asserts"][0]["value"]


def test_update_force_two_atoms_kat():
    """solver/src/lib.rs:91-107 (default particle mass 1)."""
    from moldyn_gb300.core import ParticleDatabase, State
    from moldyn_gb300.solver import PotentialsDatabase, set_precision, update_force
    set_precision("fp64")
    ParticleDatabase.add(0, "test_particle", 1.0, 0.1)
    counts, pos, vel, mass, box = rc.two_atoms_at_rest()
    st = State(pos, vel, [0, 0], box)
    update_force(PotentialsDatabase(), st)
    for a in rc.kats()["update_force_lennard_jones"]["asserts"]:
        assert rc.fmt8(st.forces[0, "xyz".index(a["expr"][-1])]) == a["value"]


# --------------------------------------------------------------------------
# force parity on synthetic systems

SYSTEMS = {
    "fcc_4x4x4": lambda: gs.fcc((4, 4, 4), jitter=0.05, seed=1),          # 256 atoms, L = 6.7 (brute)
    "fcc_6x6x6": lambda: gs.fcc((6, 6, 6), jitter=0.08, seed=2),          # 864 atoms, cells
    "fcc_8x8x10": lambda: gs.fcc((8, 8, 10), jitter=0.06, seed=3),        # 2560 atoms, cells
    "gas_small_box": lambda: gs.gas(60, (4.5, 4.5, 4.5), seed=4),        # L < 2 r_cut
    "gas_sparse": lambda: gs.gas(400, (20.0, 20.0, 20.0), seed=5),
}


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_fp64_reference_order_forces_bitexact(mdgb, oracle, name):
    pos, vel, box = SYSTEMS[name]()
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", ref=True)
    _upload(e, pos, vel, box)
    e.compute_forces()
    out = e.download()
    assert np.array_equal(out["force"], ost.force)
    assert np.array_equal(out["potential"], ost.potential)
    assert np.array_equal(out["temp"], ost.temp)
    e.close()


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_pair_set_equals_all_pairs(mdgb, oracle, name):
    """Cell binning + Verlet list select exactly the reference's pair set."""
    pos, vel, box = SYSTEMS[name]()
    ost = _oracle_state(oracle, pos, vel, box)
    oi, oj = ost.pairs()
    for prec in ("fp64", "mixed"):
        e = _engine(mdgb, prec)
        _upload(e, pos, vel, box)
        e.compute_forces()
        gi, gj = e.interacting_pairs()
        assert len(gi) == len(oi)
        assert set(zip(gi.tolist(), gj.tolist())) == set(zip(oi.tolist(), oj.tolist()))
        e.close()


@pytest.mark.parametrize("name", sorted(SYSTEMS))
@pytest.mark.parametrize("tpa", [1, 2, 4, 8])
def test_fp64_tree_order_forces(mdgb, oracle, name, tpa):
    """FP64 plain path, any threads-per-atom: <= 1e-12 of the force scale."""
    pos, vel, box = SYSTEMS[name]()
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", threads_per_atom=tpa)
    _upload(e, pos, vel, box)
    e.compute_forces()
    out = e.download()
    scale = np.abs(ost.force).max()
    assert np.abs(out["force"] - ost.force).max() <= 1e-12 * scale
    assert np.abs(out["potential"] - ost.potential).max() <= 1e-12 * np.abs(ost.potential).max()
    assert np.abs(out["temp"] - ost.temp).max() <= 1e-12 * np.abs(ost.temp).max()
    e.close()


@pytest.mark.parametrize("name", sorted(SYSTEMS))
@pytest.mark.parametrize("tpa", [1, 2, 4, 8])
def test_mixed_forces_error(mdgb, oracle, name, tpa):
    """Mixed path: per-atom relative force error <= 1e-5 (floored at the rms
    force) and rms error <= 3e-6 of the rms force; per-atom potential within
    1e-5 of its scale."""
    pos, vel, box = SYSTEMS[name]()
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "mixed", threads_per_atom=tpa)
    _upload(e, pos, vel, box)
    e.compute_forces()
    out = e.download()
    fmag = np.sqrt((ost.force ** 2).sum(axis=1))
    rms = np.sqrt((fmag ** 2).mean())
    err = np.sqrt(((out["force"] - ost.force) ** 2).sum(axis=1))
    # per-atom relative error, floored at the rms force (atoms with ~zero net force)
    rel_max, rel_rms = (err / np.maximum(fmag, rms)).max(), np.sqrt((err ** 2).mean()) / rms
    print(f"{name} tpa={tpa}: max {rel_max:.3e} rms {rel_rms:.3e}")
    assert rel_max <= 1e-5 and rel_rms <= 3e-6, (rel_max, rel_rms)
    assert np.abs(out["potential"] - ost.potential).max() <= 1e-5 * np.abs(ost.potential).max()
    e.close()


def _cutoff_pairs():
    """Isolated pairs whose separations straddle r_cut = 2.5 sigma by a few
    parts in 1e7..1e6 (inside the mixed path's 1e-5 band, where FP32 cannot
    decide), along an axis and along a diagonal, 7 sigma apart."""
    deltas = [-3e-6, -1e-6, -2e-7, 0.0, 2e-7, 1e-6, 3e-6]
    dirs = [np.array([1.0, 0.0, 0.0]), np.array([1.0, 1.0, 1.0]) / np.sqrt(3.0)]
    pos = []
    k = 0
    for dv in dirs:
        for dl in deltas:
            g = np.array([k % 4, (k // 4) % 4, k // 16], dtype=np.float64) * 7.0 + 1.0
            pos.append(g)
            pos.append(g + dv * 2.5 * (1.0 + dl))
            k += 1
    pos = np.array(pos)
    box = np.array([28.0, 28.0, 28.0])
    vel = np.zeros_like(pos)
    return pos, vel, box


@pytest.mark.parametrize("tpa", [1, 2, 8])
def test_mixed_pairs_at_the_cutoff(mdgb, oracle, tpa):
    """Pairs within 1e-5 of r_cut^2 are decided with the reference's FP64
    arithmetic (k_force_band): the mixed path includes exactly the pairs the
    oracle includes, with forces to the mixed bar, also through fused steps."""
    pos, vel, box = _cutoff_pairs()
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "mixed", threads_per_atom=tpa)
    _upload(e, pos, vel, box)
    e.compute_forces()
    out = e.download()
    on = np.linalg.norm(ost.force, axis=1) > 0
    gn = np.linalg.norm(out["force"], axis=1) > 0
    assert on.any() and (~on).any()          # both sides of the cutoff are present
    assert np.array_equal(on, gn)
    assert np.allclose(out["force"], ost.force, rtol=1e-5, atol=1e-7 * np.abs(ost.force).max())
    # fused NVE steps carry the band atoms' kick and drift too
    e.step(30, 0.005)
    ost.step(0.005, nsteps=30)
    got = e.download()
    assert np.allclose(got["pos"], ost.pos, rtol=0, atol=1e-9)
    assert np.allclose(got["vel"], ost.vel, rtol=0, atol=1e-8)
    e.close()


def test_multitype_reference_semantics(mdgb, oracle):
    """Two types with their own LJ pairs; atoms of type t see only types >= t
    (potential.rs:171-176), bit-identical in reference order."""
    pos, vel, box = gs.fcc((5, 5, 5), jitter=0.05, seed=9)
    n = len(pos)
    types = (np.arange(n) % 3 == 0).astype(np.uint16)
    order = np.argsort(types, kind="stable")      # oracle wants type-major order
    pairs = {(0, 0): (1.0, 1.0), (0, 1): (1.1, 0.8), (1, 1): (0.9, 1.3)}
    ost = oracle.OracleState([int((types == 0).sum()), int((types == 1).sum())], pos[order], vel[order],
                             [1.0, 2.0], box, oracle.pot_table(2, pairs))
    ost.update_force()
    e = _engine(mdgb, "fp64", ref=True)
    for (a, b), (s, ep) in pairs.items():
        e.set_potential(a, b, s, ep)
    e.upload(types, pos, vel, [1.0, 2.0], box)
    e.compute_forces()
    out = e.download()
    assert np.array_equal(out["force"][order], ost.force)
    assert np.array_equal(out["potential"][order], ost.potential)
    e.close()


# --------------------------------------------------------------------------
# trajectories

def test_nve_trajectory_reference_order_bitexact(mdgb, oracle):
    pos, vel, box = gs.fcc((5, 5, 5), jitter=0.03, seed=11)
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", ref=True)
    _upload(e, pos, vel, box)
    e.compute_forces()
    for chunk in (1, 7, 42):
        e.step(chunk, 0.005)
        ost.step(0.005, nsteps=chunk)
        out = e.download()
        assert np.array_equal(out["pos"], ost.pos)
        assert np.array_equal(out["vel"], ost.vel)
        assert np.array_equal(out["force"], ost.force)
    e.close()


def test_berendsen_thermostat_reference_order_bitexact(mdgb, oracle):
    from moldyn_gb300.initializer import Thermostat
    pos, vel, box = gs.fcc((5, 5, 5), jitter=0.03, seed=12, t_star=1.2)
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", ref=True)
    _upload(e, pos, vel, box)
    e.compute_forces()
    th = Thermostat.Berendsen(0.5)
    oth = oracle.Thermostat(oracle.BERENDSEN, 0.5, 0.0, 0.0)
    T0 = gs.t_ref(0.72)
    for chunk in (1, 30):
        e.step(chunk, 0.005, thermostat=th, target_temperature=T0)
        ost.step(0.005, nsteps=chunk, thermostat=oth, T0=T0)
        out = e.download()
        assert th.lambda_ == oth.lambda_
        assert np.array_equal(out["pos"], ost.pos) and np.array_equal(out["vel"], ost.vel)
    e.close()


@pytest.mark.parametrize("ref", [True, False])
def test_nose_hoover_trajectory(mdgb, oracle, ref):
    """Nose-Hoover (thermostat.rs:35-39,59-65): psi advances with the
    temperature before the first kick and again with the temperature between
    kick and scaling.  lambda = exp(.) uses CUDA's exp against the C library's
    (they may differ by an ulp), so the bar is 1e-10 after 40 steps."""
    from moldyn_gb300.initializer import Thermostat
    pos, vel, box = gs.fcc((5, 5, 5), jitter=0.03, seed=17, t_star=1.1)
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", ref=ref)
    _upload(e, pos, vel, box)
    e.compute_forces()
    th = Thermostat.NoseHoover(0.4)
    oth = oracle.Thermostat(oracle.NOSE_HOOVER, 0.4, 0.0, 0.0)
    T0 = gs.t_ref(0.72)
    for chunk in (1, 39):
        e.step(chunk, 0.005, thermostat=th, target_temperature=T0)
        ost.step(0.005, nsteps=chunk, thermostat=oth, T0=T0)
        out = e.download()
        assert abs(th.psi - oth.psi) <= 1e-12 * max(1.0, abs(oth.psi))
        assert abs(th.lambda_ - oth.lambda_) <= 1e-14
        assert np.abs(out["pos"] - ost.pos).max() <= 1e-10
        assert np.abs(out["vel"] - ost.vel).max() <= 1e-10
    assert oth.psi != 0.0
    e.close()


def test_berendsen_barostat_trajectory(mdgb, oracle):
    """Barostat: mu = cbrt(.) uses CUDA's cbrt against the C library's, so a
    1-ulp difference per step is allowed; trajectories agree to 1e-11."""
    from moldyn_gb300.initializer import Barostat, Thermostat
    pos, vel, box = gs.fcc((5, 5, 5), jitter=0.03, seed=13)
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", ref=True)
    _upload(e, pos, vel, box)
    e.compute_forces()
    ba, th = Barostat.Berendsen(1.0, 5.0), Thermostat.Berendsen(0.5)
    oba, oth = oracle.Barostat(1.0, 5.0, 0.0), oracle.Thermostat(oracle.BERENDSEN, 0.5, 0.0, 0.0)
    T0 = gs.t_ref(0.72)
    e.step(40, 0.005, thermostat=th, target_temperature=T0, barostat=ba, target_pressure=1.0)
    ost.step(0.005, nsteps=40, barostat=oba, P0=1.0, thermostat=oth, T0=T0)
    out = e.download()
    assert abs(ba.myu - oba.myu) <= 1e-14
    assert np.allclose(out["box"], ost.box, rtol=1e-12, atol=0)
    assert np.abs(out["pos"] - ost.pos).max() <= 1e-11 * ost.box.max()
    assert np.abs(out["vel"] - ost.vel).max() <= 1e-9
    e.close()


def test_fp64_tree_trajectory_close(mdgb, oracle):
    pos, vel, box = gs.fcc((6, 6, 6), jitter=0.03, seed=14)
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", threads_per_atom=4)
    _upload(e, pos, vel, box)
    e.compute_forces()
    e.step(60, 0.005)
    ost.step(0.005, nsteps=60)
    out = e.download()
    assert np.abs(out["pos"] - ost.pos).max() <= 1e-9
    e.close()


def test_mixed_trajectory_close(mdgb, oracle):
    """Short mixed trajectory stays within 1e-5 of the FP64 oracle."""
    pos, vel, box = gs.fcc((6, 6, 6), jitter=0.03, seed=15)
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "mixed")
    _upload(e, pos, vel, box)
    e.compute_forces()
    e.step(20, 0.005)
    ost.step(0.005, nsteps=20)
    out = e.download()
    d = out["pos"] - ost.pos
    d -= box * np.round(d / box)
    assert np.abs(d).max() <= 1e-5
    m = e.macro(0)
    assert abs(m["kinetic_energy"] - ost.kinetic_energy()) <= 1e-5 * ost.kinetic_energy()
    e.close()


def test_macro_tree_mode_matches_oracle(mdgb, oracle):
    pos, vel, box = gs.fcc((6, 6, 6), jitter=0.05, seed=16)
    vel = vel + np.array([0.3, -0.1, 0.2])     # non-zero COM velocity
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64")
    _upload(e, pos, vel, box)
    e.compute_forces()
    m = e.macro(0)
    assert np.allclose(m["com_velocity"], ost.com_velocity(), rtol=1e-13, atol=1e-15)
    for k, v in (("kinetic_energy", ost.kinetic_energy()), ("thermal_energy", ost.thermal_energy()),
                 ("potential_energy", ost.potential_energy()), ("pressure", ost.pressure()),
                 ("temperature", ost.temperature())):
        assert abs(m[k] - v) <= 1e-12 * abs(v), k
    e.close()


# --------------------------------------------------------------------------
# ensembles, recovery, determinism

def test_ensemble_matches_each_replica(mdgb, oracle):
    """Independent replicas of uneven size and density in one engine: each is
    bit-identical to its own oracle run (FP64 reference order, thermostat)."""
    from moldyn_gb300.initializer import Thermostat
    systems = [gs.fcc((2, 2, 2), seed=20), gs.fcc((5, 4, 3), jitter=0.05, seed=21),
               gs.gas(90, (9.0, 9.0, 9.0), seed=22), gs.fcc((6, 6, 6), rho=0.6, seed=23)]
    offs = np.cumsum([0] + [len(s[0]) for s in systems])
    pos = np.concatenate([s[0] for s in systems])
    vel = np.concatenate([s[1] for s in systems])
    boxes = np.array([s[2] for s in systems])
    e = _engine(mdgb, "fp64", ref=True)
    e.set_potential(0, 0, 1.0, 1.0)
    e.upload_ensemble(offs, np.zeros(len(pos), dtype=np.uint16), pos, vel, [1.0], boxes)
    e.compute_forces()
    T0s = [gs.t_ref(t) for t in (0.6, 0.9, 1.5, 2.0)]
    ths = [Thermostat.Berendsen(0.5) for _ in systems]
    e.ensemble_set_coupling(ths, T0s)
    e.ensemble_step(25, 0.005)
    e.ensemble_get_coupling()
    out = e.download()
    for r, (p, v, b) in enumerate(systems):
        ost = _oracle_state(oracle, p, v, b)
        ost.update_force()
        oth = oracle.Thermostat(oracle.BERENDSEN, 0.5, 0.0, 0.0)
        ost.step(0.005, nsteps=25, thermostat=oth, T0=T0s[r])
        sl = slice(offs[r], offs[r + 1])
        assert np.array_equal(out["pos"][sl], ost.pos), r
        assert np.array_equal(out["vel"][sl], ost.vel), r
        assert ths[r].lambda_ == oth.lambda_
    e.close()


def test_neighbor_overflow_recovers(mdgb, oracle):
    """A list capacity far too small is detected on the device, grown, and the
    chunk re-run: results equal an engine that never overflowed."""
    pos, vel, box = gs.fcc((6, 6, 6), jitter=0.03, seed=30)
    ost = _oracle_state(oracle, pos, vel, box)
    ost.update_force()
    e = _engine(mdgb, "fp64", ref=True, neighbor_capacity=8)
    _upload(e, pos, vel, box)
    e.compute_forces()
    e.step(10, 0.005)
    ost.step(0.005, nsteps=10)
    out = e.download()
    assert np.array_equal(out["pos"], ost.pos)
    s = e.stats()
    assert s.neighbor_capacity > 8
    e.close()


def test_fixed_point_overflow_is_reported(mdgb):
    """Nearly overlapping atoms push a pair force past the fixed-point range:
    the mixed path returns MDGB_ERR_FIXED_POINT_OVERFLOW (no device fault)."""
    from moldyn_gb300 import _lib
    pos = np.array([[1.0, 1.0, 1.0], [1.02, 1.0, 1.0], [3.0, 3.0, 3.0]])
    e = _engine(mdgb, "mixed")
    _upload(e, pos, np.zeros((3, 3)), (6.0, 6.0, 6.0))
    with pytest.raises(_lib.MdgbError) as ei:
        e.compute_forces()
    assert ei.value.status == 5
    e.close()


@pytest.mark.parametrize("kw", [{}, dict(graph_steps=10)])
def test_nve_chunk_leaves_current_forces_potential_and_temp(mdgb, kw):
    """The fused passes of an NVE chunk store neither forces nor per-atom
    potential and temp; the chunk's last pass must leave all three as a fresh
    evaluation at the final positions gives them.  A fresh engine bins the
    atoms anew (other cell centres, so other FP32 roundings): compared at the
    mixed bar, 1e-5 of the rms -- values one step old are off by ~1e-2."""
    pos, vel, box = gs.fcc((8, 8, 8), jitter=0.04, seed=33)
    e = _engine(mdgb, "mixed", threads_per_atom=1, **kw)
    _upload(e, pos, vel, box)
    e.compute_forces()
    e.step(30, 0.005)
    out = e.download()
    e.close()
    f = _engine(mdgb, "mixed", threads_per_atom=1)
    _upload(f, out["pos"], out["vel"], box)
    f.compute_forces()
    fresh = f.download()
    f.close()
    for k in ("force", "potential", "temp"):
        scale = np.sqrt(np.mean(fresh[k] ** 2))
        assert np.max(np.abs(out[k] - fresh[k])) <= 1e-5 * scale, k


def test_mixed_is_deterministic(mdgb):
    pos, vel, box = gs.fcc((8, 8, 8), jitter=0.04, seed=31)
    outs = []
    for _ in range(2):
        e = _engine(mdgb, "mixed", threads_per_atom=4)
        _upload(e, pos, vel, box)
        e.compute_forces()
        e.step(30, 0.005)
        outs.append(e.download())
        e.close()
    for k in ("pos", "vel", "force", "potential", "temp"):
        assert np.array_equal(outs[0][k], outs[1][k]), k


@pytest.mark.parametrize("opts", [dict(graph_steps=10), dict(persistent=True)])
def test_graph_and_persistent_match_eager(mdgb, opts):
    pos, vel, box = gs.fcc((8, 8, 8), jitter=0.04, seed=32)
    outs, graph_launches = [], []
    for kw in ({}, opts):
        e = _engine(mdgb, "mixed", threads_per_atom=2, **kw)
        _upload(e, pos, vel, box)
        e.compute_forces()
        e.step(30, 0.005)
        outs.append(e.download())
        graph_launches.append(e.stats().graph_launches)
        e.close()
    for k in ("pos", "vel", "force"):
        assert np.array_equal(outs[0][k], outs[1][k]), k
    assert graph_launches[1] > 0 if "graph_steps" in opts else True


def test_argon_berendsen_tp_reference_units(mdgb, oracle):
    """The argon configuration in the reference's units (U lattice 10^3, edge
    3.338339 nm, m 66.335, sigma 0.3405 nm, eps/kB 119.8 K, Berendsen tau 10 ->
    300 K, barostat (1, 5) -> 1.01325, dt 0.002): FP64 reference order against
    the oracle over 200 steps.  Thermostat factors agree bit for bit; the
    barostat's cbrt may differ by an ulp per step (CUDA vs C library)."""
    from moldyn_gb300.initializer import Barostat, Thermostat, UnitCell, lattice_positions, maxwell_boltzmann
    a, m, sig, eps = 3.338339, 66.335, 0.3405, 119.8 * gs.K_B * 0.01
    pos = lattice_positions(UnitCell.U, (10, 10, 10), a)
    vel = maxwell_boltzmann(1000, 273.15, m, 7)
    box = np.full(3, 10 * a)
    e = _engine(mdgb, "fp64", ref=True)
    _upload(e, pos, vel, box, mass=m, sigma=sig, eps=eps)
    e.compute_forces()
    th, ba = Thermostat.Berendsen(10.0), Barostat.Berendsen(1.0, 5.0)
    e.step(200, 0.002, thermostat=th, target_temperature=300.0, barostat=ba, target_pressure=1.01325)
    out = e.download()
    e.close()
    ost = _oracle_state(oracle, pos, vel, box, mass=m, sigma=sig, eps=eps)
    ost.update_force()
    oth, oba = oracle.Thermostat(oracle.BERENDSEN, 10.0, 0.0, 0.0), oracle.Barostat(1.0, 5.0, 0.0)
    ost.step(0.002, nsteps=200, barostat=oba, P0=1.01325, thermostat=oth, T0=300.0)
    assert abs(th.lambda_ - oth.lambda_) <= 1e-14 and abs(ba.myu - oba.myu) <= 1e-14
    assert np.allclose(out["box"], ost.box, rtol=1e-13, atol=0)
    assert np.abs(out["pos"] - ost.pos).max() <= 1e-10
    assert np.abs(out["vel"] - ost.vel).max() <= 1e-10


def test_download_preserves_caller_order(mdgb):
    pos, vel, box = gs.fcc((6, 6, 6), jitter=0.04, seed=33)
    perm = np.random.default_rng(0).permutation(len(pos))
    e = _engine(mdgb, "fp64")
    _upload(e, pos[perm], vel[perm], box)
    e.compute_forces()                         # rebuild sorts atoms by cell on the device
    out = e.download()
    assert np.array_equal(out["pos"], pos[perm]) and np.array_equal(out["vel"], vel[perm])
    e.close()


def test_ieee_conversions_match_cuda(tmp_path):
    """The integer-op double<->float conversions the drift and force kernels
    use agree with CUDA's conversion instructions bit for bit."""
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "conv_check")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                           os.path.join(root, "tests", "cuda", "conv_check.cu"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr


def test_trace_phases_account_for_the_step_kernel(mdgb):
    """MDGB_FLAG_TRACE: per-phase device time of the step kernel; launch and
    rebuild counts match the steps taken and the rebuild statistics."""
    pos, vel, box = gs.fcc((8, 8, 8), jitter=0.02, seed=31)
    e = _engine(mdgb, "mixed", trace=True)
    _upload(e, pos, vel, box)
    e.compute_forces()
    e.trace_phases()                      # reset
    e.reset_stats()
    e.step(40, 0.005)
    ph = e.trace_phases()
    st = e.stats()
    assert ph["launches"] == 40
    assert ph["rebuild_launches"] == st.rebuilds
    assert all(v >= 0.0 for v in ph.values())
    if st.rebuilds:
        assert ph["verlet_list"] > 0.0 and ph["gather"] > 0.0
    assert e.trace_phases()["launches"] == 0  # read-and-reset
    e.close()


def test_fp64_rate_probe(tmp_path):
    """The DFMA throughput the FP64 path's pipe fraction is quoted against
    (tests/cuda/dfma_rate.cu): a plausible rate for GB300's FP64 pipe."""
    import os
    import re
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "dfma_rate")
    subprocess.check_call(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                           os.path.join(root, "tests", "cuda", "dfma_rate.cu"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    per_clk = float(re.search(r"per SM per clk at \d+ MHz: ([0-9.]+)", out.stdout).group(1))
    print(out.stdout.strip())
    assert 0.5 < per_clk < 4.0 and "err=no error" in out.stdout
