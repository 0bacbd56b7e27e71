"""Mirror of moldyn_solver::macro_parameters (solver/src/macro_parameters/*.rs).

Each reduction runs on the GPU (FP64) over the State's device copy:
get_center_of_mass_velocity (mod.rs:12-25), get_momentum_of_system
(mod.rs:28-34), get_kinetic_energy / get_thermal_energy /
get_potential_energy (energy.rs:14-49), get_pressure (pressure.rs:5-20).
get_temperature (temperature.rs:4-7) is the reference's scalar formula.
"""
from __future__ import annotations

import numpy as np

from .core import K_B, State
from .solver import _engine_for


def _macro(state: State, particle_type_id: int) -> dict:
    return _engine_for(None, state).macro(particle_type_id)


def get_center_of_mass_velocity(state: State, particle_type_id: int) -> np.ndarray:
    return _macro(state, particle_type_id)["com_velocity"]


def get_momentum_of_system(state: State, particle_type_id: int) -> np.ndarray:
    return _macro(state, particle_type_id)["momentum"]


def get_kinetic_energy(state: State, particle_type_id: int) -> float:
    return _macro(state, particle_type_id)["kinetic_energy"]


def get_thermal_energy(state: State, particle_type_id: int, center_of_mass_velocity=None) -> float:
    """The reference passes get_center_of_mass_velocity(state, t) here; the GPU
    reduction computes that same centre-of-mass velocity itself."""
    return _macro(state, particle_type_id)["thermal_energy"]


def get_potential_energy(state: State, particle_type_id: int) -> float:
    return _macro(state, particle_type_id)["potential_energy"]


def get_pressure(state: State, particle_type_id: int, center_of_mass_velocity=None) -> float:
    return _macro(state, particle_type_id)["pressure"]


def get_temperature(thermal_energy: float, number_particles: int) -> float:
    """temperature.rs:4-7: 2E / (3 N K_B), scaled x100 to kelvin."""
    t = (2.0 * thermal_energy) / (3.0 * float(number_particles) * K_B)
    return t * 100.0
