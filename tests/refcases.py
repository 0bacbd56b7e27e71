"""Initial conditions of the reference's own unit tests, shared by the oracle
golden tests (CPU) and the GPU parity tests.

Each builder returns (counts, pos, vel, mass_per_type, box) in the flat
type-major layout.  `Particle::default()` has mass 1.0 (core/src/particle.rs:
78-91); the two-atom systems set mass 66.335 explicitly.
"""
from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_kats.json")


def kats():
    with open(GOLDEN) as f:
        return json.load(f)["tests"]


def two_atoms_at_rest():
    """solver/src/lib.rs:91-107: (0,0,0) and (0.5,0,0), box 2, default mass 1."""
    pos = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])
    vel = np.zeros((2, 3))
    return np.array([2]), pos, vel, np.array([1.0]), np.array([2.0, 2.0, 2.0])


def two_argon_moving():
    """solver/src/lib.rs:109-125 (also :264-280, :334-348, :379-393, :404-418,
    and cli/src/tests.rs:35-56)."""
    pos = np.array([[0.75, 0.75, 0.5], [1.25, 0.75, 0.5]])
    vel = np.array([[1.0, 1.0, 0.0], [-1.0, 1.0, 0.0]])
    return np.array([2]), pos, vel, np.array([66.335]), np.array([2.0, 2.0, 2.0])


def fmt8(x: float) -> str:
    """Rust `format!("{:.8}", x)`: correctly rounded fixed notation."""
    return format(float(x), ".8f")


def lattice_argon_8():
    """solver/src/lib.rs:59-68: 8 argon atoms on a 2x2x2 U lattice, edge 3.338339."""
    a = 3.338339
    pos = np.array([[x * a, y * a, z * a] for x in range(2) for y in range(2) for z in range(2)],
                   dtype=np.float64)
    return pos, np.array([2.0 * a, 2.0 * a, 2.0 * a])
