"""Headless particle render -- the GUI viewer's frame without a window.

Mirrors gui/src/visualizer/camera.rs (Camera, get_right_up) and
CameraUniform::from (window.rs:366-377: cgmath look_to_rh and perspective with
near 0.01, far 10000), builds the GUI's per-particle instance data
(ParticleDataLite, window.rs:53-57, :340-350) from a State, and renders through
``mdgb_splat`` (moldyn_gb300/csrc/splat.cu): spheres ray-cast on the GPU and
shaded as shader.wgsl, box edges as bounding_box.wgsl.  The image is an
(height, width, 4) float32 array, row 0 at the top; ``write_ppm`` stores it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .core import ParticleDatabase, State

F32 = np.float32

# window.rs:466-472: the viewer's initial visualisation parameters
DEFAULT_GRADIENT = ((0.0, 0.0, 0.0, 1.0), (0.5, 0.5, 0.5, 1.0), (1.0, 1.0, 1.0, 1.0))
MODE_TYPE = 0
MODE_SPEED = 1


def _norm(v: np.ndarray) -> np.ndarray:
    v = np.asarray(v, dtype=F32)
    return (v * (F32(1.0) / F32(np.sqrt(np.dot(v, v))))).astype(F32)


class Camera:
    """camera.rs:3-60 (eye, fovy in degrees, forward, right, up, screen size)."""

    def __init__(self, eye=(-1.0, 0.0, 0.0), fovy: float = 70.0, width: int = 1920, height: int = 1080,
                 forward=(1.0, 0.0, 0.0)):
        self.eye = np.array(eye, dtype=F32)
        self.fovy = F32(fovy)
        self.update(eye, forward, width, height)

    def update(self, eye, forward, width: int, height: int):
        """Camera::update (camera.rs:42-60)."""
        self.eye = np.array(eye, dtype=F32)
        self.forward = _norm(forward)
        self.width, self.height = int(width), int(height)
        self.right, self.up = self._right_up()

    def _right_up(self):
        """get_right_up (camera.rs:13-26): world up is -y."""
        world_up = np.array([0.0, -1.0, 0.0], dtype=F32)
        right = _norm(np.cross(self.forward, world_up))
        up = _norm(np.cross(self.forward, right))
        up_length = F32(np.tan(np.radians(self.fovy) / 2.0))
        right_length = F32(up_length / F32(self.height / self.width))
        return (right * right_length).astype(F32), (up * up_length).astype(F32)

    def uniform(self):
        """CameraUniform::from (window.rs:366-377): view_pos, column-major view
        (look_to_rh(eye, forward, up)) and projection (perspective)."""
        f = _norm(self.forward)
        s = _norm(np.cross(f, self.up))
        u = np.cross(s, f).astype(F32)
        e = self.eye
        view = np.array([s[0], u[0], -f[0], 0.0,
                         s[1], u[1], -f[1], 0.0,
                         s[2], u[2], -f[2], 0.0,
                         -np.dot(e, s), -np.dot(e, u), np.dot(e, f), 1.0], dtype=F32)
        aspect = F32(self.width) / F32(self.height)
        near, far = F32(0.01), F32(10000.0)
        fc = F32(1.0) / F32(np.tan(np.radians(self.fovy) / 2.0))
        proj = np.zeros(16, dtype=F32)
        proj[0] = fc / aspect
        proj[5] = fc
        proj[10] = (far + near) / (near - far)
        proj[11] = -1.0
        proj[14] = (F32(2.0) * far * near) / (near - far)
        view_pos = np.array([e[0], e[1], e[2], 1.0], dtype=F32)
        return view_pos, view, proj


def framing_camera(box, width: int, height: int, fovy: float = 70.0) -> Camera:
    """A camera on the -x side of the box looking along +x (the viewer's
    initial direction, camera.rs:28-30) far enough back to see all of it."""
    box = np.asarray(box, dtype=np.float64)
    half = 0.5 * max(box[1], box[2] * height / width if width else box[2])   # screen up = y, right = z
    dist = half / np.tan(np.radians(fovy) / 2.0) * 1.1 + 0.5 * box[0]
    centre = 0.5 * box
    return Camera(eye=(centre[0] - dist, centre[1], centre[2]), fovy=fovy, width=width, height=height)


def particle_data(state: State) -> np.ndarray:
    """ParticleDataLite::from for every particle (window.rs:340-350), in the
    state's order: (x, y, z, 1), (vx, vy, vz, 1), (mass, radius, id, 0)."""
    n = state.n
    out = np.zeros((n, 12), dtype=F32)
    out[:, 0:3] = state.positions
    out[:, 3] = 1.0
    out[:, 4:7] = state.velocities
    out[:, 7] = 1.0
    for t in np.unique(state.ids):
        sel = state.ids == t
        m, r = ParticleDatabase.get_particle_mass(int(t)), ParticleDatabase.get_particle_radius(int(t))
        if m is None or r is None:
            raise KeyError(f"particle id {int(t)} is not in ParticleDatabase")
        out[sel, 8] = m
        out[sel, 9] = r
        out[sel, 10] = float(t)
    return out


def splat_params(camera: Camera, mode: int = MODE_TYPE, gradient=DEFAULT_GRADIENT, speed_range=(0.0, 1.0),
                 box=None) -> _lib.CSplatParams:
    view_pos, view, proj = camera.uniform()
    p = _lib.CSplatParams()
    p.view_pos[:] = [float(x) for x in view_pos]
    p.view[:] = [float(x) for x in view]
    p.proj[:] = [float(x) for x in proj]
    p.gradient_min[:] = [float(x) for x in gradient[0]]
    p.gradient_mid[:] = [float(x) for x in gradient[1]]
    p.gradient_max[:] = [float(x) for x in gradient[2]]
    p.gradient_min_max[:] = [float(speed_range[0]), float(speed_range[1]), 0.0, 0.0]
    p.mode = int(mode)
    if box is not None:
        p.draw_box = 1
        p.box[:] = [float(box[0]), float(box[1]), float(box[2]), 0.0]
    return p


def splat(particles: np.ndarray, params: _lib.CSplatParams, width: int, height: int) -> np.ndarray:
    """mdgb_splat: (height, width, 4) float32 RGBA."""
    parts = np.ascontiguousarray(particles, dtype=F32).reshape(-1, 12)
    out = np.zeros((height, width, 4), dtype=F32)
    L = _lib.load()
    rc = L.mdgb_splat(parts, parts.shape[0], C.byref(params), int(width), int(height), out)
    if rc != _lib.MDGB_OK:
        raise _lib.MdgbError(rc, "mdgb_splat failed")
    return out


def render_state(state: State, camera: Camera | None = None, width: int = 640, height: int = 360,
                 mode: int = MODE_TYPE, gradient=DEFAULT_GRADIENT, speed_range=(0.0, 1.0),
                 draw_box: bool = True) -> np.ndarray:
    cam = camera or framing_camera(state.boundary_box, width, height)
    cam.update(cam.eye, cam.forward, width, height)
    params = splat_params(cam, mode, gradient, speed_range, state.boundary_box if draw_box else None)
    return splat(particle_data(state), params, width, height)


def write_ppm(path: str, rgba: np.ndarray):
    """Binary PPM (P6) of the RGB channels, clamped to [0, 1]."""
    h, w = rgba.shape[:2]
    rgb = np.clip(rgba[:, :, :3], 0.0, 1.0)
    data = np.round(rgb * 255.0).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode())
        f.write(data.tobytes())


def read_ppm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        raw = f.read()
    parts = raw.split(b"\n", 3)
    w, h = (int(x) for x in parts[1].split())
    return np.frombuffer(parts[3], dtype=np.uint8).reshape(h, w, 3)
