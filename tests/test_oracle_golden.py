"""Pin the oracle to the reference's own golden test values.

Every assert in tests/golden/reference_kats.json (extracted from
solver/src/lib.rs and cli/src/tests.rs) is reproduced by the oracle to the
same 8-decimal string the reference test compares.
"""
from __future__ import annotations

import numpy as np
import pytest

from tests import refcases as rc

DEFAULT_TABLE = None


def _table(o):
    return o.pot_table(1)


def _quantities(o, st):
    """Names used by the reference tests for the two-atom systems."""
    q = {}
    for k, name in ((0, "1"), (1, "2")):
        for a, ax in enumerate("xyz"):
            q[f"pos{name}.{ax}"] = st.pos[k, a]
            q[f"v{name}.{ax}"] = st.vel[k, a]
            q[f"f{name}.{ax}"] = st.force[k, a]
    mv = st.com_velocity(0)
    kin = st.kinetic_energy(0)
    th = st.thermal_energy(0, mv)
    pe = st.potential_energy(0)
    q.update({"kinetic": kin, "e_kinetic": kin, "thermal": th, "e_thermal": th,
              "potential": pe, "e_potential": pe, "internal": th + pe, "e_internal": th + pe,
              "full": kin + pe, "e": kin + pe,
              "temperature": o.temperature(th, 2),
              "temperature / 100.0": o.temperature(th, 2) / 100.0,
              "pressure": st.pressure(0, mv), "mv": mv})
    return q


def _check_asserts(o, st, asserts, step_fn):
    done = 0
    checked = 0
    for a in sorted(asserts, key=lambda r: r["after_steps"]):
        while done < a["after_steps"]:
            step_fn(st)
            done += 1
        q = _quantities(o, st)
        if "value" in a:
            got = rc.fmt8(q[a["expr"]])
            assert got == a["value"], f"{a['source']}: {a['expr']} = {got}, reference {a['value']}"
        else:
            assert a["expr"] == "mv"
            assert tuple(q["mv"]) == (0.0, 1.0, 0.0), a["source"]
        checked += 1
    return checked


def test_lennard_jones(oracle):
    """solver/src/lib.rs:77-89."""
    pot = oracle.lj_new(0.3418, 1.712)
    u, f = oracle.lj_eval(pot, 0.5)
    want = {a["expr"]: a["value"] for a in rc.kats()["lennard_jones"]["asserts"]}
    assert rc.fmt8(u) == want["potential"]
    assert rc.fmt8(f) == want["force"]


def test_update_force_two_atoms(oracle):
    """solver/src/lib.rs:91-107."""
    counts, pos, vel, mass, box = rc.two_atoms_at_rest()
    st = oracle.OracleState(counts, pos, vel, mass, box, _table(oracle))
    st.update_force()
    for a in rc.kats()["update_force_lennard_jones"]["asserts"]:
        ax = "xyz".index(a["expr"][-1])
        assert rc.fmt8(st.force[0, ax]) == a["value"], a["source"]


@pytest.mark.parametrize("name", ["verlet_with_lennard_jones", "verlet_lj_1000_iterations",
                                  "energies", "temperature", "pressure", "solvation"])
def test_two_argon_kats(oracle, name):
    """solver/src/lib.rs:109-427 and cli/src/tests.rs:35-98: the two-argon
    trajectory (NVE, dt 0.002) and its macro parameters."""
    counts, pos, vel, mass, box = rc.two_argon_moving()
    st = oracle.OracleState(counts, pos, vel, mass, box, _table(oracle))
    st.update_force()
    n = _check_asserts(oracle, st, rc.kats()[name]["asserts"], lambda s: s.step(0.002))
    assert n == len(rc.kats()[name]["asserts"]) and n > 0


def test_initialization_box_and_count(oracle):
    """cli/src/tests.rs:9-33: 10^3 U argon lattice, edge 3.338339."""
    want = {a["expr"]: a["equals"] for a in rc.kats()["initialization"]["asserts"]}
    pos = oracle.lattice("U", 10, 10, 10, 3.338339)
    assert len(pos) == int(want["state.particles[0].len()"])
    box = 3.338339 * 10.0
    assert box == float(want["state.boundary_box.x"])


def test_lattice_index_order(oracle):
    """solver/src/lib.rs:17-47: U lattice index x*ny*nz + y*nz + z."""
    pos = oracle.lattice("U", 2, 2, 2, 2.0)
    assert tuple(pos[2]) == (0.0, 2.0, 0.0)


def test_fcc_sites(oracle):
    """solver/src/initializer/position.rs:55-99: 4 sites per cell."""
    pos = oracle.lattice("FCC", 1, 1, 2, 1.0)
    want = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                     [0, 0, 1], [0, .5, 1.5], [.5, 0, 1.5], [.5, .5, 1]], dtype=float)
    assert np.array_equal(pos, want)


def test_momentum_conserved_property(oracle):
    """solver/src/lib.rs:59-75 (shortened to 2000 steps): the +/- velocity
    pairing gives zero momentum, and NVE Verlet keeps |sum v| < 1e-12."""
    pos, box = rc.lattice_argon_8()
    rng = np.random.default_rng(5)
    half = rng.normal(size=(4, 3)) * np.sqrt(oracle.K_B * 273.15 * 0.01 / 66.335)
    vel = np.concatenate([half, -half])
    st = oracle.OracleState([8], pos, vel, [66.335], box, _table(oracle))
    st.update_force()
    for _ in range(20):
        st.step(0.002, nsteps=100)
        p = st.vel.sum(axis=0)
        assert np.all(np.abs(p) < 1e-12)


def test_thread_count_independent(oracle):
    """rayon only distributes rows: results are bit-identical for any thread count."""
    rng = np.random.default_rng(1)
    n = 300
    box = np.array([3.0, 3.0, 3.0])
    pos = rng.random((n, 3)) * box
    a = oracle.OracleState([n], pos, np.zeros((n, 3)), [1.0], box, _table(oracle))
    b = oracle.OracleState([n], pos, np.zeros((n, 3)), [1.0], box, _table(oracle))
    a.update_force(nthreads=1)
    b.update_force(nthreads=4)
    assert np.array_equal(a.force, b.force) and np.array_equal(a.temp, b.temp)
