"""ctypes wrapper around the oracle library (test infrastructure only).

The oracle is a CPU FP64 restatement of the moldyn solver path (see
``oracle/mdref.cpp`` for the file:line map).  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module; the product package ``moldyn_gb300`` never does.

States are flat, type-major numpy arrays: ``counts[t]`` atoms of type ``t``
follow those of type ``t-1``, which is the order the reference's
``StateToSave::from`` flattens ``Vec<Vec<Particle>>`` into.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build  # type: ignore

_LIB = None

K_B = 1.380648528  # core/src/lib.rs:15

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class Thermostat(C.Structure):
    """Mirror of ``Thermostat`` (solver/src/initializer/thermostat.rs:4-20)."""
    _fields_ = [("kind", C.c_int), ("tau", C.c_double), ("lambda_", C.c_double),
                ("psi", C.c_double)]


class Barostat(C.Structure):
    """Mirror of ``Barostat::Berendsen`` (solver/src/initializer/barostat.rs:4-16)."""
    _fields_ = [("beta", C.c_double), ("tau", C.c_double), ("myu", C.c_double)]


BERENDSEN = 0
NOSE_HOOVER = 1


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = C.CDLL(path)
        L.oref_lj_new.argtypes = [C.c_double, C.c_double, _dp]
        L.oref_lj_eval.argtypes = [_dp, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oref_update_force.argtypes = [C.c_int, _ip, _dp, _dp, _dp, _dp, _dp, _dp,
                                        C.c_int, C.c_int64, C.c_int64]
        L.oref_update_force.restype = C.c_int
        L.oref_com_velocity.argtypes = [C.c_int, _ip, _dp, _dp, C.c_int, _dp]
        L.oref_momentum.argtypes = [C.c_int, _ip, _dp, _dp, C.c_int, _dp]
        L.oref_kinetic_energy.argtypes = [C.c_int, _ip, _dp, _dp, C.c_int]
        L.oref_kinetic_energy.restype = C.c_double
        L.oref_thermal_energy.argtypes = [C.c_int, _ip, _dp, _dp, C.c_int, _dp]
        L.oref_thermal_energy.restype = C.c_double
        L.oref_potential_energy.argtypes = [C.c_int, _ip, _dp, C.c_int]
        L.oref_potential_energy.restype = C.c_double
        L.oref_pressure.argtypes = [C.c_int, _ip, _dp, _dp, _dp, C.c_int, _dp, _dp]
        L.oref_pressure.restype = C.c_double
        L.oref_temperature.argtypes = [C.c_double, C.c_int64]
        L.oref_temperature.restype = C.c_double
        L.oref_step.argtypes = [C.c_int, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                C.c_double, C.c_int64, C.POINTER(Barostat), C.c_double,
                                C.POINTER(Thermostat), C.c_double, C.c_int]
        L.oref_step.restype = C.c_int
        L.oref_lattice.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int64, C.c_double,
                                   _dp, _dp]
        L.oref_apply_boundary_conditions.argtypes = [C.c_int64, _dp, _dp]
        L.oref_pairs.argtypes = [C.c_int, _ip, _dp, _dp, _dp, C.c_int64,
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.oref_pairs.restype = C.c_int64
        _LIB = L
    return _LIB


def lj_new(sigma: float, eps: float) -> np.ndarray:
    out = np.zeros(4)
    lib().oref_lj_new(sigma, eps, out)
    return out


def lj_eval(pot: np.ndarray, r: float):
    u, f = C.c_double(), C.c_double()
    lib().oref_lj_eval(np.ascontiguousarray(pot, dtype=np.float64), r, C.byref(u), C.byref(f))
    return u.value, f.value


def pot_table(ntypes: int, pairs: dict | None = None, default=(0.3418, 1.712)) -> np.ndarray:
    """Symmetric {sigma, eps, r_cut, u_cut} table as PotentialsDatabase builds it
    (potential.rs:95-101 default, :141-154 lookup)."""
    pairs = pairs or {}
    tab = np.zeros((ntypes, ntypes, 4))
    for a in range(ntypes):
        for b in range(ntypes):
            key = (min(a, b), max(a, b))
            s, e = pairs.get(key, default)
            tab[a, b] = lj_new(s, e)
    return np.ascontiguousarray(tab.reshape(-1))


class OracleState:
    """Flat type-major FP64 state used by the oracle."""

    def __init__(self, counts, pos, vel, mass_per_type, box, table):
        self.counts = np.ascontiguousarray(counts, dtype=np.int64)
        self.ntypes = len(self.counts)
        n = int(self.counts.sum())
        self.pos = np.ascontiguousarray(np.asarray(pos, dtype=np.float64).reshape(n, 3)).copy()
        self.vel = np.ascontiguousarray(np.asarray(vel, dtype=np.float64).reshape(n, 3)).copy()
        self.force = np.zeros((n, 3))
        self.potential = np.zeros(n)
        self.temp = np.zeros(n)
        self.mass = np.ascontiguousarray(mass_per_type, dtype=np.float64)
        self.box = np.ascontiguousarray(box, dtype=np.float64).copy()
        self.table = np.ascontiguousarray(table, dtype=np.float64)

    @property
    def n(self):
        return int(self.counts.sum())

    def update_force(self, nthreads: int = 0, rows=None):
        rb, re = (0, -1) if rows is None else rows
        lib().oref_update_force(self.ntypes, self.counts, self.pos.reshape(-1), self.box,
                                self.table, self.force.reshape(-1), self.potential, self.temp,
                                nthreads, rb, re)

    def pairs(self):
        """Interacting (i, j) pairs of update_force, flat indices."""
        n = lib().oref_pairs(self.ntypes, self.counts, self.pos.reshape(-1), self.box, self.table, 0,
                             None, None)
        ii = np.zeros(max(n, 1), dtype=np.int32)
        jj = np.zeros(max(n, 1), dtype=np.int32)
        lib().oref_pairs(self.ntypes, self.counts, self.pos.reshape(-1), self.box, self.table, n,
                         ii.ctypes.data_as(C.POINTER(C.c_int32)), jj.ctypes.data_as(C.POINTER(C.c_int32)))
        return ii[:n], jj[:n]

    def step(self, dt, nsteps=1, barostat=None, P0=0.0, thermostat=None, T0=0.0, nthreads=0):
        bp = C.pointer(barostat) if barostat is not None else None
        tp = C.pointer(thermostat) if thermostat is not None else None
        lib().oref_step(self.ntypes, self.counts, self.pos.reshape(-1), self.vel.reshape(-1),
                        self.force.reshape(-1), self.potential, self.temp, self.mass, self.box,
                        self.table, dt, nsteps, bp, P0, tp, T0, nthreads)

    def com_velocity(self, t=0):
        out = np.zeros(3)
        lib().oref_com_velocity(self.ntypes, self.counts, self.vel.reshape(-1), self.mass, t, out)
        return out

    def momentum(self, t=0):
        out = np.zeros(3)
        lib().oref_momentum(self.ntypes, self.counts, self.vel.reshape(-1), self.mass, t, out)
        return out

    def kinetic_energy(self, t=0):
        return lib().oref_kinetic_energy(self.ntypes, self.counts, self.vel.reshape(-1), self.mass, t)

    def thermal_energy(self, t=0, vcm=None):
        vcm = self.com_velocity(t) if vcm is None else np.ascontiguousarray(vcm, dtype=np.float64)
        return lib().oref_thermal_energy(self.ntypes, self.counts, self.vel.reshape(-1),
                                         self.mass, t, vcm)

    def potential_energy(self, t=0):
        return lib().oref_potential_energy(self.ntypes, self.counts, self.potential, t)

    def pressure(self, t=0, vcm=None):
        vcm = self.com_velocity(t) if vcm is None else np.ascontiguousarray(vcm, dtype=np.float64)
        return lib().oref_pressure(self.ntypes, self.counts, self.vel.reshape(-1), self.temp,
                                   self.mass, t, vcm, self.box)

    def temperature(self, t=0):
        return lib().oref_temperature(self.thermal_energy(t), int(self.counts[t]))


def temperature(thermal_energy: float, n: int) -> float:
    return lib().oref_temperature(thermal_energy, n)


def lattice(kind: str, nx: int, ny: int, nz: int, a: float, start=(0.0, 0.0, 0.0)) -> np.ndarray:
    k = 0 if kind.upper() == "U" else 1
    n = nx * ny * nz * (1 if k == 0 else 4)
    out = np.zeros(3 * n)
    lib().oref_lattice(k, nx, ny, nz, a, np.ascontiguousarray(start, dtype=np.float64), out)
    return out.reshape(n, 3)


def default_threads() -> int:
    return os.cpu_count() or 1
