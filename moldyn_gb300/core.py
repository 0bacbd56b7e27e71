"""Data model mirroring moldyn_core (core/src/particle.rs, particles_database.rs).

The reference keeps an array of structs grouped by type
(``State { particles: Vec<Vec<Particle>>, boundary_box }``,
core/src/particle.rs:5-32).  Here a State is structure-of-arrays: one flat
atom array with a type id per atom; the k-th atom of type t in flat order is
the reference's ``particles[t][k]``.  A State may carry a device-resident
engine (see solver.py) so repeated calls do not re-upload.
"""
from __future__ import annotations

import csv
import os

import numpy as np

K_B = 1.380648528  # core/src/lib.rs:15


def fmt_float(x: float) -> str:
    """Shortest round-trip decimal with Rust's exponent style ("1e-7")."""
    x = float(x)
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "inf" if x > 0 else "-inf"
    r = repr(x)
    if "e" in r:
        m, e = r.split("e")
        return f"{m}e{int(e)}"
    return r


class ParticleDatabase:
    """Process-global particle-type table (particles_database.rs:33-146):
    id -> (name, mass in 1e-27 kg, radius in nm)."""

    _data: dict[int, tuple[str, float, float]] = {}

    @classmethod
    def add(cls, id: int, name: str, mass: float, radius: float):
        cls._data[int(id)] = (str(name), float(mass), float(radius))

    @classmethod
    def get_particle_mass(cls, id: int):
        v = cls._data.get(int(id))
        return None if v is None else v[1]

    @classmethod
    def get_particle_radius(cls, id: int):
        v = cls._data.get(int(id))
        return None if v is None else v[2]

    @classmethod
    def get_particle_name(cls, id: int):
        v = cls._data.get(int(id))
        return None if v is None else v[0]

    @classmethod
    def clear_particles(cls):
        cls._data.clear()

    @classmethod
    def save_particles_data(cls, path):
        """db.csv with header id,name,mass,radius (particles_database.rs:157-194)."""
        os.makedirs(path, exist_ok=True)
        with open(os.path.join(path, "db.csv"), "w", newline="") as f:
            w = csv.writer(f, lineterminator="\n")
            w.writerow(["id", "name", "mass", "radius"])
            for i, (name, m, r) in cls._data.items():
                w.writerow([i, name, fmt_float(m), fmt_float(r)])

    @classmethod
    def load_particles_data(cls, path):
        """Loads db.csv; existing ids are kept (`or_insert`, particles_database.rs:222-224)."""
        with open(os.path.join(path, "db.csv"), newline="") as f:
            for row in csv.DictReader(f):
                i = int(row["id"])
                if i not in cls._data:
                    cls._data[i] = (row["name"], float(row["mass"]), float(row["radius"]))


class State:
    """positions/velocities/forces (N,3) float64, potential/temp (N,) float64,
    ids (N,) uint16, boundary_box (3,) float64."""

    def __init__(self, positions, velocities, ids, boundary_box, forces=None, potential=None, temp=None):
        self.positions = np.array(positions, dtype=np.float64).reshape(-1, 3)
        n = len(self.positions)
        self.velocities = (np.zeros((n, 3)) if velocities is None
                           else np.array(velocities, dtype=np.float64).reshape(n, 3))
        self.ids = np.array(ids, dtype=np.uint16).reshape(n)
        self.boundary_box = np.array(boundary_box, dtype=np.float64).reshape(3)
        self.forces = np.zeros((n, 3)) if forces is None else np.array(forces, dtype=np.float64).reshape(n, 3)
        self.potential = np.zeros(n) if potential is None else np.array(potential, dtype=np.float64).reshape(n)
        self.temp = np.zeros(n) if temp is None else np.array(temp, dtype=np.float64).reshape(n)
        self._engine = None
        self._synced = None  # host copy the device state corresponds to

    @property
    def n(self) -> int:
        return len(self.positions)

    @property
    def ntypes(self) -> int:
        return int(self.ids.max()) + 1 if self.n else 0

    def type_indices(self, particle_type_id: int) -> np.ndarray:
        """Flat indices of particles[t] in reference order."""
        return np.nonzero(self.ids == particle_type_id)[0]

    def masses_per_type(self) -> np.ndarray:
        out = []
        for t in range(self.ntypes):
            m = ParticleDatabase.get_particle_mass(t)
            if m is None:
                raise KeyError(f"particle id {t} is not in ParticleDatabase")
            out.append(m)
        return np.array(out, dtype=np.float64)

    def count(self, particle_type_id: int) -> int:
        return int(np.count_nonzero(self.ids == particle_type_id))
