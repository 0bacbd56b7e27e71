"""Mirror of moldyn_solver::solver (solver/src/solver/{potential,integrator}.rs).

Same names, arguments and error behaviour as the reference:

    pdb = PotentialsDatabase()                # default LJ(0.3418, 1.712)
    update_force(pdb, state)                  # potential.rs:158
    Integrator.VerletMethod.calculate(pdb, state, dt, barostat, thermostat)
                                              # integrator.rs:14-15
    # barostat = None or (Barostat, P0); thermostat = None or (Thermostat, T0)

Every call runs on the GPU through libmdgb: the State is uploaded (only when
its host arrays changed since the last call), the kernels run, and the
result is downloaded into the State's arrays.  The precision of these calls
is the module setting ``set_precision`` (default: FP64 in the reference's
summation order, so results are bit-identical to the reference's).
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _lib
from .core import State
from .engine import Engine

_settings = {"precision": "fp64", "reference_order": True}


def set_precision(precision: str = "fp64", reference_order: bool | None = None):
    """Choose the engine used by the functional API: "fp64" (plain path) or
    "mixed".  reference_order defaults to True for fp64."""
    if precision not in ("fp64", "mixed"):
        raise ValueError(precision)
    _settings["precision"] = precision
    _settings["reference_order"] = (precision == "fp64") if reference_order is None else reference_order


class Potential:
    """Potential::LennardJones { sigma, eps, r_cut, u_cut } (potential.rs:10-23)."""

    def __init__(self, sigma: float, eps: float, r_cut: float, u_cut: float):
        self.sigma, self.eps, self.r_cut, self.u_cut = float(sigma), float(eps), float(r_cut), float(u_cut)

    @classmethod
    def new_lennard_jones(cls, sigma: float, eps: float) -> "Potential":
        out = np.zeros(4)
        _lib.check(_lib.load().mdgb_lj_new(float(sigma), float(eps), out))
        return cls(*out)

    def params(self) -> np.ndarray:
        return np.array([self.sigma, self.eps, self.r_cut, self.u_cut])

    def get_potential_and_force(self, r: float):
        u, f = C.c_double(), C.c_double()
        _lib.check(_lib.load().mdgb_lj_eval(self.params(), float(r), C.byref(u), C.byref(f)))
        return u.value, f.value

    def get_radius_cut(self) -> float:
        return self.r_cut

    def to_serde(self) -> dict:
        return {"LennardJones": {"sigma": self.sigma, "eps": self.eps, "r_cut": self.r_cut,
                                 "u_cut": self.u_cut}}

    @classmethod
    def from_serde(cls, obj: dict) -> "Potential":
        if "LennardJones" not in obj:
            raise NotImplementedError("only LennardJones potentials are supported (Custom is todo!() "
                                      "in the reference)")
        p = obj["LennardJones"]
        return cls(p["sigma"], p["eps"], p["r_cut"], p["u_cut"])

    def __eq__(self, o):
        return isinstance(o, Potential) and np.array_equal(self.params(), o.params())


class PotentialsDatabase:
    """potential.rs:89-155: unordered (id, id) -> Potential, default LJ(0.3418, 1.712)."""

    def __init__(self):
        self.potentials: dict[tuple[int, int], Potential] = {}
        self.default_potential = Potential.new_lennard_jones(0.3418, 1.712)

    @staticmethod
    def _key(a: int, b: int):
        a, b = int(a), int(b)
        return (b, a) if a > b else (a, b)

    def set_potential(self, id0: int, id1: int, potential: Potential):
        self.potentials[self._key(id0, id1)] = potential

    def get_potential(self, id0: int, id1: int) -> Potential:
        return self.potentials.get(self._key(id0, id1), self.default_potential)

    def save_potentials_to_file(self, path):
        """potentials.json, keys "a,b" (potential.rs:104-122)."""
        os.makedirs(path, exist_ok=True)
        data = {f"{a},{b}": p.to_serde() for (a, b), p in self.potentials.items()}
        with open(os.path.join(path, "potentials.json"), "w") as f:
            json.dump(data, f, indent=2)

    def load_potentials_from_file(self, path):
        """potential.rs:125-139 (keys parsed as u16 pairs, inserted as stored)."""
        with open(os.path.join(path, "potentials.json")) as f:
            data = json.load(f)
        for key, obj in data.items():
            a, b = (int(x) for x in key.split(","))
            self.potentials[(a, b)] = Potential.from_serde(obj)


def _engine_for(pdb: PotentialsDatabase | None, state: State) -> Engine:
    """Bind `state` to a device-resident engine with `pdb`'s potentials,
    uploading only what changed since the last call.  pdb=None keeps the
    engine's potentials (the default database for a new engine)."""
    key = (_settings["precision"], _settings["reference_order"])
    eng = state._engine
    if eng is None or getattr(eng, "_key", None) != key:
        eng = Engine(precision=key[0], reference_order=key[1])
        eng._key = key
        eng._pots = None
        state._engine = eng
        state._synced = None
    ntypes = state.ntypes
    if pdb is None:
        pdb = PotentialsDatabase() if eng._pots is None else None
    pots = eng._pots if pdb is None else tuple(tuple(pdb.get_potential(a, b).params()) for a in range(ntypes) for b in range(a, ntypes))
    if eng._pots != pots:
        i = 0
        for a in range(ntypes):
            for b in range(a, ntypes):
                eng.set_potential_raw(a, b, *pots[i])
                i += 1
        eng._pots = pots
    masses = state.masses_per_type()
    snap = state._synced
    fresh = (snap is None or snap["n"] != state.n or not np.array_equal(snap["ids"], state.ids)
             or not np.array_equal(snap["masses"], masses)
             or not np.array_equal(snap["pos"], state.positions)
             or not np.array_equal(snap["vel"], state.velocities)
             or not np.array_equal(snap["box"], state.boundary_box))
    if fresh:
        eng.upload(state.ids, state.positions, state.velocities, masses, state.boundary_box)
        eng.upload_forces(state.forces, state.potential, state.temp)
    elif not (np.array_equal(snap["force"], state.forces) and np.array_equal(snap["potential"], state.potential)
              and np.array_equal(snap["temp"], state.temp)):
        eng.upload_forces(state.forces, state.potential, state.temp)
    return eng


def _pull(eng: Engine, state: State):
    out = eng.download()
    state.positions[...] = out["pos"]
    state.velocities[...] = out["vel"]
    state.forces[...] = out["force"]
    state.potential[...] = out["potential"]
    state.temp[...] = out["temp"]
    state.boundary_box[...] = out["box"]
    state._synced = {"n": state.n, "ids": state.ids.copy(), "masses": state.masses_per_type(),
                     "pos": state.positions.copy(), "vel": state.velocities.copy(),
                     "box": state.boundary_box.copy(), "force": state.forces.copy(),
                     "potential": state.potential.copy(), "temp": state.temp.copy()}


def update_force(potentials_database: PotentialsDatabase, state: State):
    """Setup potentials and forces for each particle in `state` (potential.rs:157-216)."""
    eng = _engine_for(potentials_database, state)
    eng.compute_forces()
    _pull(eng, state)


class Integrator:
    """Integrator::VerletMethod / Integrator::Custom (integrator.rs:5-11)."""

    def __init__(self, kind: str = "verlet", name: str | None = None):
        self.kind = kind
        self.name = name

    @classmethod
    def Custom(cls, name: str) -> "Integrator":
        return cls("custom", name)

    def calculate(self, potentials_database: PotentialsDatabase, state: State, delta_time: float,
                  barostat=None, thermostat=None, steps: int = 1):
        """integrator.rs:14-59, `steps` times.  barostat = (Barostat, P0) or None;
        thermostat = (Thermostat, T0) or None; their fields are updated in place."""
        if self.kind != "verlet":
            raise NotImplementedError("Integrator::Custom is todo!() in the reference")
        eng = _engine_for(potentials_database, state)
        th, t0 = thermostat if thermostat is not None else (None, 0.0)
        ba, p0 = barostat if barostat is not None else (None, 0.0)
        eng.step(steps, delta_time, thermostat=th, target_temperature=t0, barostat=ba, target_pressure=p0)
        _pull(eng, state)


Integrator.VerletMethod = Integrator("verlet")
