"""Initializers and coupling objects, mirroring moldyn_solver::initializer.

Thermostat / Barostat mirror solver/src/initializer/thermostat.rs:4-20 and
barostat.rs:4-16 (the enum variants and their mutable fields).  Lattice and
velocity set-up call libmdgb's host helpers (mdgb_lattice,
mdgb_maxwell_boltzmann); they run once, before the hot loop.
"""
from __future__ import annotations

import enum

import numpy as np

from . import _lib
from .core import ParticleDatabase, State


class InitError(Exception):
    """solver/src/initializer/position.rs:10-14."""


class ParticleIdDidNotFound(InitError):
    pass


class TooBig(InitError):
    pass


class OutOfBoundary(InitError):
    pass


class UnitCell(enum.Enum):
    U = 0
    FCC = 1


class Thermostat:
    """Thermostat::Berendsen { tau, lambda } / NoseHoover { tau, psi, lambda }."""

    def __init__(self, kind: str, tau: float, lambda_: float = 0.0, psi: float = 0.0):
        if kind not in ("berendsen", "nose_hoover"):
            raise ValueError(kind)
        self.kind = kind
        self.tau = float(tau)
        self.lambda_ = float(lambda_)
        self.psi = float(psi)

    @property
    def kind_id(self) -> int:
        return _lib.THERMOSTAT_BERENDSEN if self.kind == "berendsen" else _lib.THERMOSTAT_NOSE_HOOVER

    @classmethod
    def Berendsen(cls, tau: float, lambda_: float = 0.0):
        return cls("berendsen", tau, lambda_)

    @classmethod
    def NoseHoover(cls, tau: float, psi: float = 0.0, lambda_: float = 0.0):
        return cls("nose_hoover", tau, lambda_, psi)


class Barostat:
    """Barostat::Berendsen { beta, tau, myu }."""

    def __init__(self, beta: float, tau: float, myu: float = 0.0):
        self.beta = float(beta)
        self.tau = float(tau)
        self.myu = float(myu)

    @classmethod
    def Berendsen(cls, beta: float, tau: float, myu: float = 0.0):
        return cls(beta, tau, myu)


def lattice_positions(unit_cell: UnitCell, grid_size, unit_cell_size: float, start=(0.0, 0.0, 0.0)):
    """Sites in the order of position.rs:34-99 (index x*ny*nz + y*nz + z)."""
    nx, ny, nz = (int(g) for g in grid_size)
    per = 1 if unit_cell == UnitCell.U else 4
    out = np.zeros(3 * nx * ny * nz * per)
    _lib.check(_lib.load().mdgb_lattice(unit_cell.value, nx, ny, nz, float(unit_cell_size),
                                        np.ascontiguousarray(start, dtype=np.float64), out))
    return out.reshape(-1, 3)


def maxwell_boltzmann(n: int, temperature: float, mass: float, seed: int) -> np.ndarray:
    """Seeded counterpart of velocity.rs:6-29: sigma = sqrt(K_B T 0.01 / m);
    first n/2 atoms +v, next n/2 -v (zero momentum)."""
    out = np.zeros(3 * n)
    _lib.check(_lib.load().mdgb_maxwell_boltzmann(int(n), float(temperature), float(mass),
                                                  int(seed) & 0xFFFFFFFFFFFFFFFF, out))
    return out.reshape(n, 3)


def initialize_particles(number_particles, boundary) -> State:
    """position.rs:116-137: zero positions/velocities, `number_particles[i]` atoms of id i."""
    ids = []
    for t, cnt in enumerate(number_particles):
        if ParticleDatabase.get_particle_mass(t) is None:
            raise ParticleIdDidNotFound(t)
        ids.extend([t] * int(cnt))
    n = len(ids)
    return State(np.zeros((n, 3)), np.zeros((n, 3)), np.array(ids, dtype=np.uint16),
                 np.asarray(boundary, dtype=np.float64))


def initialize_particles_position(unit_cell: UnitCell, state: State, particle_id: int, start_position,
                                  grid_size, unit_cell_size: float):
    """position.rs:155-174 and the UnitCell fill (:25-99)."""
    if ParticleDatabase.get_particle_mass(particle_id) is None:
        raise ParticleIdDidNotFound(particle_id)
    box = state.boundary_box
    if any(g * unit_cell_size > b for g, b in zip(grid_size, box)):
        raise OutOfBoundary()
    idx = np.nonzero(state.ids == particle_id)[0]
    per = 1 if unit_cell == UnitCell.U else 4
    need = int(np.prod(grid_size)) * per
    if need > len(idx):
        raise TooBig()
    sites = lattice_positions(unit_cell, grid_size, unit_cell_size, start_position)
    state.positions[idx[:need]] = sites


def initialize_velocities_maxwell_boltzmann(state: State, temperature: float, particle_id: int,
                                            seed: int = 0):
    mass = ParticleDatabase.get_particle_mass(particle_id)
    if mass is None:
        raise ParticleIdDidNotFound(particle_id)
    idx = np.nonzero(state.ids == particle_id)[0]
    state.velocities[idx] = maxwell_boltzmann(len(idx), temperature, mass, seed)
