"""moldyn_gb300 -- GB300-native molecular-dynamics step engine.

A drop-in for moldyn's force / neighbour / integration path (Lennard-Jones,
velocity Verlet, Berendsen thermostat and barostat).  The compute runs in
hand-written sm_103a CUDA kernels in libmdgb.so (C ABI: include/mdgb.h);
this package is the Python host side mirroring the reference's crates:

    moldyn_gb300.core              moldyn_core (State, ParticleDatabase, K_B)
    moldyn_gb300.solver            moldyn_solver::solver (Potential, PotentialsDatabase,
                                   update_force, Integrator)
    moldyn_gb300.initializer       moldyn_solver::initializer (Thermostat, Barostat, lattices,
                                   Maxwell-Boltzmann)
    moldyn_gb300.macro_parameters  moldyn_solver::macro_parameters
    moldyn_gb300.engine            the persistent device-resident Engine (performance API)
"""
from . import _lib
from .core import K_B, ParticleDatabase, State
from .engine import Engine

__all__ = ["Engine", "State", "ParticleDatabase", "K_B", "lib_path", "load_library"]


def lib_path() -> str:
    return _lib.lib_path()


def load_library():
    """Load (building if needed) libmdgb.so; raises if it cannot be built."""
    return _lib.load()
