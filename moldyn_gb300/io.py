"""State / frame / macro-parameter files, in the reference's formats.

A simulation directory holds (core/src/save_data.rs:155-230,
core/src/particles_database.rs:157-228, solver/src/solver/potential.rs:104-139):

    bb.csv            x,y,z           one row per frame (the box of frame n is row n)
    data/<n>.csv      id,position_x,position_y,position_z,velocity_x,velocity_y,velocity_z
    db.csv            id,name,mass,radius
    potentials.json   {"a,b": {"LennardJones": {"sigma", "eps", "r_cut", "u_cut"}}}
    macro.csv         iteration,kinetic_energy,potential_energy,thermal_energy,
                      unit_kinetic_energy,unit_potential_energy,unit_thermal_energy,
                      temperature,pressure,custom

Floats are written in shortest round-trip form with the exponent style of
Rust's float formatting ("1e-7", "1.5e20"), so files written here read back
bit-exactly, here and in the reference.
"""
from __future__ import annotations

import csv
import os
import queue
import threading

import numpy as np

from .core import ParticleDatabase, State, fmt_float

FRAME_HEADER = ["id", "position_x", "position_y", "position_z", "velocity_x", "velocity_y", "velocity_z"]
MACRO_HEADER = ["iteration", "kinetic_energy", "potential_energy", "thermal_energy", "unit_kinetic_energy",
                "unit_potential_energy", "unit_thermal_energy", "temperature", "pressure", "custom"]


def _rows(path):
    with open(path, newline="") as f:
        return list(csv.DictReader(f))


def load_boxes(directory) -> list:
    p = os.path.join(directory, "bb.csv")
    if not os.path.exists(p):
        return []
    return [np.array([float(r["x"]), float(r["y"]), float(r["z"])]) for r in _rows(p)]


def save_boxes(directory, boxes):
    with open(os.path.join(directory, "bb.csv"), "w", newline="") as f:
        f.write("x,y,z\n")
        for b in boxes:
            f.write(",".join(fmt_float(v) for v in b) + "\n")


def save_frame(directory, frame: int, ids, positions, velocities):
    """data/<frame>.csv in flat (type-major) order, like StateToSave::from."""
    d = os.path.join(directory, "data")
    os.makedirs(d, exist_ok=True)
    ids = np.asarray(ids)
    pos = np.asarray(positions, dtype=np.float64)
    vel = np.asarray(velocities, dtype=np.float64)
    lines = [",".join(FRAME_HEADER)]
    for i in range(len(ids)):
        p, v = pos[i], vel[i]
        lines.append(f"{int(ids[i])},{fmt_float(p[0])},{fmt_float(p[1])},{fmt_float(p[2])},"
                     f"{fmt_float(v[0])},{fmt_float(v[1])},{fmt_float(v[2])}")
    with open(os.path.join(d, f"{frame}.csv"), "w", newline="") as f:
        f.write("\n".join(lines) + "\n")


class FrameWriter:
    """save_frame on a background thread, so formatting a frame's CSV overlaps
    the device's next steps (the engine's calls release the interpreter lock
    while the GPU works).  Frames are written in submission order; at most
    `depth` wait in the queue (submit blocks beyond that).  A write error is
    raised by the next submit or by close."""

    def __init__(self, directory, depth: int = 2):
        self.directory = directory
        self._q: queue.Queue = queue.Queue(maxsize=max(1, depth))
        self._error: BaseException | None = None
        self._thread = threading.Thread(target=self._run, name="frame-writer", daemon=True)
        self._thread.start()

    def _run(self):
        while True:
            item = self._q.get()
            try:
                if item is None:
                    return
                if self._error is None:
                    save_frame(self.directory, *item)
            except BaseException as exc:  # reported on the caller's thread
                self._error = exc
            finally:
                self._q.task_done()

    def _raise(self):
        if self._error is not None:
            err, self._error = self._error, None
            raise err

    def submit(self, frame: int, ids, positions, velocities):
        """Queue data/<frame>.csv; the arrays must not be modified afterwards."""
        self._raise()
        if not self._thread.is_alive():
            raise RuntimeError("frame writer is closed")
        self._q.put((frame, ids, positions, velocities))

    def close(self):
        """Write every queued frame, stop the thread, raise a pending error."""
        if self._thread.is_alive():
            self._q.put(None)
            self._thread.join()
        self._raise()

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc, tb):
        if exc_type is None:
            self.close()
        elif self._thread.is_alive():
            self._q.put(None)
            self._thread.join()


def save_state(directory, frame: int, state: State):
    """StateToSave::save_to_file (save_data.rs:192-213): the frame file and row
    `frame` of bb.csv (replaced if present, else appended)."""
    os.makedirs(directory, exist_ok=True)
    boxes = load_boxes(directory)
    if len(boxes) > frame:
        boxes[frame] = state.boundary_box.copy()
    else:
        boxes.append(state.boundary_box.copy())
    save_boxes(directory, boxes)
    order = np.argsort(state.ids, kind="stable")
    save_frame(directory, frame, state.ids[order], state.positions[order], state.velocities[order])


def load_state(directory, frame: int) -> State:
    """StateToSave::load_from_file + Into<State> (save_data.rs:129-151, 215-229):
    atoms grouped by id in file order; masses from the ParticleDatabase."""
    boxes = load_boxes(directory)
    rows = _rows(os.path.join(directory, "data", f"{frame}.csv"))
    ids = np.array([int(r["id"]) for r in rows], dtype=np.uint16)
    pos = np.array([[float(r["position_x"]), float(r["position_y"]), float(r["position_z"])] for r in rows])
    vel = np.array([[float(r["velocity_x"]), float(r["velocity_y"]), float(r["velocity_z"])] for r in rows])
    order = np.argsort(ids, kind="stable")
    return State(pos[order].reshape(-1, 3), vel[order].reshape(-1, 3), ids[order], boxes[frame])


def frame_numbers(directory) -> list:
    d = os.path.join(directory, "data")
    return sorted(int(f[:-4]) for f in os.listdir(d) if f.endswith(".csv") and f[:-4].isdigit())


def save_macro(directory, rows: list):
    """DataFileMacro::save_to_file (save_data.rs:291-300), rows sorted by iteration."""
    with open(os.path.join(directory, "macro.csv"), "w", newline="") as f:
        f.write(",".join(MACRO_HEADER) + "\n")
        for r in sorted(rows, key=lambda q: q["iteration"]):
            f.write(str(int(r["iteration"])) + "," + ",".join(fmt_float(r[k]) for k in MACRO_HEADER[1:]) + "\n")


def load_macro(directory) -> list:
    out = []
    for r in _rows(os.path.join(directory, "macro.csv")):
        q = {k: float(v) for k, v in r.items()}
        q["iteration"] = int(r["iteration"])
        out.append(q)
    return out


def save_particles(directory):
    ParticleDatabase.save_particles_data(directory)


def load_particles(directory):
    ParticleDatabase.load_particles_data(directory)
