"""The moldyn-cli drop-in (moldyn_gb300/cli.py) and the reference's file formats."""
from __future__ import annotations

import os

import numpy as np
import pytest

from tests import refcases as rc


def _cli(*argv):
    from moldyn_gb300.cli import main
    main(list(argv))


def test_fmt_float_round_trips():
    from moldyn_gb300.core import fmt_float
    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.standard_normal(2000) * 10.0 ** rng.integers(-30, 30, 2000),
                           [0.0, -0.0, 1.0, 1e-7, 1.5e20, 33.38339, 0.75]])
    for v in vals:
        s = fmt_float(v)
        assert float(s) == v and "+" not in s
    assert fmt_float(1e-7) == "1e-7" and fmt_float(1.5e20) == "1.5e20" and fmt_float(2.0) == "2.0"


def test_cli_initialization_kat(tmp_path):
    """cli/src/tests.rs:9-33: 10^3 U argon -> 1000 atoms, box 33.38339, db entry."""
    from moldyn_gb300 import io as mio
    from moldyn_gb300.core import ParticleDatabase
    d = str(tmp_path)
    _cli("-f", d, "initialize", "-t", "u", "-s", "10", "10", "10", "-n", "Argon", "-m", "66.335",
         "-r", "0.071", "-l", "3.338339", "-T", "273.15")
    ParticleDatabase.clear_particles()
    mio.load_particles(d)
    want = {a["expr"]: a["equals"] for a in rc.kats()["initialization"]["asserts"]}
    assert ParticleDatabase.get_particle_name(0) == want["name"].strip('"')
    assert ParticleDatabase.get_particle_mass(0) == float(want["mass"])
    assert ParticleDatabase.get_particle_radius(0) == float(want["radius"])
    st = mio.load_state(d, 0)
    assert st.n == int(want["state.particles[0].len()"])
    assert st.boundary_box[0] == float(want["state.boundary_box.x"])
    assert np.all(np.abs(st.velocities.sum(axis=0)) < 1e-12)   # +/- pairing: zero momentum


def test_frame_and_box_files(tmp_path):
    from moldyn_gb300 import io as mio
    from moldyn_gb300.core import ParticleDatabase, State
    ParticleDatabase.add(0, "a", 1.0, 0.1)
    ParticleDatabase.add(1, "b", 2.0, 0.2)
    d = str(tmp_path)
    st = State([[0.1, 0.2, 0.3], [1.0, 1.1, 1.2], [2.0, 2.1, 2.2]], [[1, 2, 3], [4, 5, 6], [7, 8, 9]],
               [1, 0, 1], [5.0, 6.0, 7.0])
    mio.save_state(d, 0, st)
    st.boundary_box[:] = [8.0, 8.0, 8.0]
    mio.save_state(d, 1, st)
    st.boundary_box[:] = [9.0, 9.0, 9.0]
    mio.save_state(d, 0, st)           # replaces row 0
    boxes = mio.load_boxes(d)
    assert [b[0] for b in boxes] == [9.0, 8.0]
    back = mio.load_state(d, 1)
    # grouped by id, file order inside a type (save_data.rs:129-151)
    assert back.ids.tolist() == [0, 1, 1]
    assert np.array_equal(back.positions, np.array([[1.0, 1.1, 1.2], [0.1, 0.2, 0.3], [2.0, 2.1, 2.2]]))
    assert open(os.path.join(d, "data", "1.csv")).readline().strip() == \
        "id,position_x,position_y,position_z,velocity_x,velocity_y,velocity_z"


def test_potentials_json_round_trip(tmp_path):
    from moldyn_gb300.solver import Potential, PotentialsDatabase
    d = str(tmp_path)
    _cli("-f", d, "generate-default-potentials")
    _cli("-f", d, "set-potential", "-i", "0", "1", "-p", "lennard-jones", "--params", "0.3405", "1.654017")
    pdb = PotentialsDatabase()
    pdb.load_potentials_from_file(d)
    assert pdb.get_potential(1, 0) == Potential.new_lennard_jones(0.3405, 1.654017)
    assert pdb.get_potential(0, 0) == Potential.new_lennard_jones(0.3418, 1.712)
    assert pdb.get_potential(1, 1) == pdb.default_potential


@pytest.mark.gpu
def test_cli_solvation_kat(tmp_path):
    """cli/src/tests.rs:35-98: two argon atoms saved as state 0, solve 3 steps
    through the frame files, reload frame 3, update_force: golden values."""
    from moldyn_gb300 import io as mio
    from moldyn_gb300.core import ParticleDatabase, State
    from moldyn_gb300.solver import PotentialsDatabase, set_precision, update_force
    d = str(tmp_path)
    ParticleDatabase.clear_particles()
    ParticleDatabase.add(0, "Argon", 66.335, 0.071)
    _, pos, vel, _, box = rc.two_argon_moving()
    mio.save_state(d, 0, State(pos, vel, [0, 0], box))
    ParticleDatabase.save_particles_data(d)
    _cli("-f", d, "solve", "-s", "0", "-i", "verlet-method", "-c", "3", "-t", "0.002")
    assert sorted(mio.frame_numbers(d)) == [0, 1, 2, 3]
    st = mio.load_state(d, 3)
    set_precision("fp64")
    update_force(PotentialsDatabase(), st)
    q = {f"pos{k + 1}.{ax}": st.positions[k, i] for k in range(2) for i, ax in enumerate("xyz")}
    q.update({f"v{k + 1}.{ax}": st.velocities[k, i] for k in range(2) for i, ax in enumerate("xyz")})
    q.update({f"f{k + 1}.{ax}": st.forces[k, i] for k in range(2) for i, ax in enumerate("xyz")})
    for a in rc.kats()["solvation"]["asserts"]:
        assert rc.fmt8(q[a["expr"]]) == a["value"], a["source"]


@pytest.mark.gpu
def test_cli_solve_with_coupling_and_macro(tmp_path, oracle):
    """solve with Berendsen T/P and --frames-per-save, then
    solve-macro-parameters -A; every frame's macro row equals the oracle's
    numbers for the same frame (temperature over all particles,
    commands.rs:233,259)."""
    from moldyn_gb300 import io as mio
    from moldyn_gb300.core import K_B, ParticleDatabase
    d = str(tmp_path)
    ParticleDatabase.clear_particles()
    _cli("-f", d, "initialize", "-t", "fcc", "-s", "3", "3", "3", "-n", "Argon", "-m", "66.335", "-r", "0.071",
         "-l", "0.5406", "-T", "120", "--seed", "4")
    _cli("-f", d, "--frames-per-save", "5", "solve", "-s", "0", "-i", "verlet-method", "-c", "20", "-t", "0.002",
         "--thermostat", "berendsen", "--thermostat-params", "1.0", "-T", "100",
         "--barostat", "berendsen", "--barostat-params", "1", "5", "-P", "20")
    frames = mio.frame_numbers(d)
    assert frames == [0, 5, 10, 15, 20]
    _cli("-f", d, "solve-macro-parameters", "-A")
    rows = {r["iteration"]: r for r in mio.load_macro(d)}
    assert sorted(rows) == frames
    for f in frames:
        st = mio.load_state(d, f)
        ost = oracle.OracleState([st.n], st.positions, st.velocities, [66.335], st.boundary_box,
                                 oracle.pot_table(1))
        ost.update_force()
        th = ost.thermal_energy()
        want = {"kinetic_energy": ost.kinetic_energy(), "potential_energy": ost.potential_energy(),
                "thermal_energy": th, "pressure": ost.pressure(),
                "temperature": (2.0 * th) / (3.0 * st.n * K_B) * 100.0}
        for k, v in want.items():
            assert rows[f][k] == v, (f, k, rows[f][k], v)


def test_frame_writer_matches_save_frame(tmp_path):
    """FrameWriter (background thread) writes the same bytes as save_frame,
    every submitted frame, in order."""
    from moldyn_gb300 import io as mio
    rng = np.random.default_rng(8)
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    frames = [(k, rng.integers(0, 3, 50), rng.standard_normal((50, 3)), rng.standard_normal((50, 3)))
              for k in range(5)]
    with mio.FrameWriter(a, depth=1) as w:
        for f in frames:
            w.submit(*f)
    for f in frames:
        mio.save_frame(b, *f)
    for k in range(5):
        with open(os.path.join(a, "data", f"{k}.csv"), "rb") as fa, \
                open(os.path.join(b, "data", f"{k}.csv"), "rb") as fb:
            assert fa.read() == fb.read()


def test_frame_writer_reports_write_errors(tmp_path):
    from moldyn_gb300 import io as mio
    blocker = tmp_path / "data"
    blocker.write_text("a file where the data directory should be")
    w = mio.FrameWriter(str(tmp_path))
    w.submit(0, np.zeros(2, dtype=int), np.zeros((2, 3)), np.zeros((2, 3)))
    with pytest.raises(OSError):
        w.close()


class _FakeEngine:
    """Stands in for the device engine: moves every atom by (step count) x dt
    along x, so each saved frame is predictable."""

    def __init__(self):
        self.steps = 0

    def set_potential_raw(self, *a):
        pass

    def upload(self, ids, pos, vel, masses, box):
        self.pos, self.vel, self.box = np.array(pos), np.array(vel), np.array(box, dtype=float)

    def compute_forces(self):
        pass

    def step(self, n, dt, **kw):
        self.steps += n
        self.pos[:, 0] += n * dt

    def download(self):
        return {"pos": self.pos.copy(), "vel": self.vel.copy(), "force": np.zeros_like(self.pos),
                "potential": np.zeros(len(self.pos)), "temp": np.zeros(len(self.pos)), "box": self.box.copy()}

    def close(self):
        pass


@pytest.mark.parametrize("fps", [1, 3])
def test_solve_loop_saves_every_frame(tmp_path, monkeypatch, fps):
    """commands.rs:258-367 bookkeeping with --frames-per-save, through the
    background frame writer (device engine replaced by a stand-in)."""
    from moldyn_gb300 import cli
    from moldyn_gb300 import io as mio
    from moldyn_gb300.core import ParticleDatabase, State
    d = str(tmp_path)
    ParticleDatabase.clear_particles()
    ParticleDatabase.add(0, "Argon", 66.335, 0.071)
    _, pos, vel, _, box = rc.two_argon_moving()
    mio.save_state(d, 0, State(pos, vel, [0, 0], box))
    ParticleDatabase.save_particles_data(d)
    fake = _FakeEngine()
    monkeypatch.setattr(cli, "_make_engine", lambda args: fake)
    _cli("-f", d, "--frames-per-save", str(fps), "solve", "-s", "0", "-i", "verlet-method", "-c", "7",
         "-t", "0.5")
    assert fake.steps == 7
    want = [0] + [k for k in range(1, 7) if k % fps == 0] + [7]
    assert sorted(mio.frame_numbers(d)) == want
    for k in want:
        st = mio.load_state(d, k)
        assert np.allclose(st.positions[:, 0], pos[:, 0] + 0.5 * k)
    assert len(mio.load_boxes(d)) == 8
