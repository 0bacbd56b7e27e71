"""Seeded synthetic systems for GPU parity tests (reduced LJ units: sigma =
eps = mass = 1).  Shapes follow the configurations the engine is measured on:
FCC lattices at rho* = 0.8442 with Maxwell-Boltzmann velocities, scaled down
so the O(N^2) oracle finishes in seconds."""
from __future__ import annotations

import numpy as np

K_B = 1.380648528


def t_ref(t_star: float) -> float:
    """Reduced temperature -> the reference's kelvin units (sigma=eps=m=1):
    K_B * T * 0.01 = T*."""
    return t_star * 100.0 / K_B


def fcc(cells, rho=0.8442, jitter=0.0, seed=0, t_star=0.72):
    """cells = (nx, ny, nz) FCC unit cells -> (pos, vel, box)."""
    cells = np.asarray(cells)
    a = (4.0 / rho) ** (1.0 / 3.0)
    g = np.stack(np.meshgrid(*[np.arange(c) for c in cells], indexing="ij"), -1).reshape(-1, 3)
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    pos = ((g[:, None, :] + basis[None]) * a).reshape(-1, 3)
    box = cells * a
    rng = np.random.default_rng(seed)
    if jitter:
        pos = np.mod(pos + rng.normal(scale=jitter, size=pos.shape), box)
    n = len(pos)
    half = rng.normal(scale=np.sqrt(t_star), size=(n // 2, 3))
    vel = np.zeros((n, 3))
    vel[: n // 2] = half
    vel[n // 2: 2 * (n // 2)] = -half
    return pos, vel, box.astype(np.float64)


def gas(n, box, seed=0, min_dist=0.9, t_star=1.0):
    """Random non-overlapping positions (rejection sampling) in a box."""
    rng = np.random.default_rng(seed)
    box = np.asarray(box, dtype=np.float64)
    pos = np.zeros((n, 3))
    k = 0
    tries = 0
    while k < n:
        tries += 1
        assert tries < 200 * n
        p = rng.random(3) * box
        d = pos[:k] - p
        d -= box * np.round(d / box)
        if k == 0 or np.min(np.einsum("ij,ij->i", d, d)) >= min_dist ** 2:
            pos[k] = p
            k += 1
    vel = rng.normal(scale=np.sqrt(t_star), size=(n, 3))
    vel -= vel.mean(axis=0)
    return pos, vel, box
