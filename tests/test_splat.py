"""Headless render (moldyn_gb300/csrc/splat.cu, mdgb_splat) against the CPU
restatement of the GUI viewer's shaders (oracle/splat_ref.py).

CPU tests pin the oracle to hand-derived values of shader.wgsl /
bounding_box.wgsl and the camera matrices to cgmath's formulas; GPU tests
require the kernel's image to equal the oracle's bit for bit (both use the same
IEEE float32 operations in the same order)."""
from __future__ import annotations

import math
import os

import numpy as np
import pytest

from oracle import splat_ref


def _params(cam, mode=0, box=None, grange=(0.0, 1.0), gradient=None):
    from moldyn_gb300 import render as rnd
    view_pos, view, proj = cam.uniform()
    return {"view_pos": view_pos, "view": view, "proj": proj, "mode": mode, "box": box, "grange": grange,
            "gradient": gradient or rnd.DEFAULT_GRADIENT}


def _scene(seed, n, box=4.0):
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 12), dtype=np.float32)
    p[:, 0:3] = rng.uniform(0.2, box - 0.2, (n, 3))
    p[:, 3] = 1.0
    p[:, 4:7] = rng.normal(0.0, 0.6, (n, 3))
    p[:, 7] = 1.0
    p[:, 8] = 1.0
    p[:, 9] = rng.uniform(0.12, 0.35, n)
    p[:, 10] = rng.integers(0, 8, n)
    return p


def test_camera_matrices_follow_cgmath():
    """look_to_rh and perspective (window.rs:366-377) for the viewer's initial
    camera: eye (-1, 0, 0), forward +x, world up -y (camera.rs:13-40)."""
    from moldyn_gb300.render import Camera
    cam = Camera((-1.0, 0.0, 0.0), 70.0, 200, 100)
    view_pos, view, proj = cam.uniform()
    # right = f x (0,-1,0) = (0,0,-1); up = f x right = (0,1,0); s = f x up = (0,0,1); u = s x f = (0,1,0)
    want_view = [0, 0, -1, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0, 0, -1, 1]
    assert np.allclose(view, want_view, atol=1e-7)
    f = 1.0 / math.tan(math.radians(35.0))
    assert proj[0] == pytest.approx(f / 2.0, rel=1e-6) and proj[5] == pytest.approx(f, rel=1e-6)
    assert proj[10] == pytest.approx((10000.01) / (0.01 - 10000.0), rel=1e-6) and proj[11] == -1.0
    assert proj[14] == pytest.approx(2 * 10000.0 * 0.01 / (0.01 - 10000.0), rel=1e-6)
    assert list(view_pos) == [-1.0, 0.0, 0.0, 1.0]


def test_oracle_single_sphere_shading():
    """A unit sphere 5 ahead of the camera: the ray through the central pixel
    hits it head-on, n = -forward; shader.wgsl:121-130 by hand."""
    from moldyn_gb300.render import Camera
    cam = Camera((0.0, 0.0, 0.0), 70.0, 65, 65)
    p = np.zeros((1, 12), dtype=np.float32)
    p[0, 0:4] = [5.0, 0.0, 0.0, 1.0]
    p[0, 9] = 1.0
    p[0, 10] = 0.0     # id 0: red
    img = splat_ref.render(p, _params(cam), 65, 65)
    n = np.array([-1.0, 0.0, 0.0])
    light = -np.array([1.0, -1.0, 1.0]) / math.sqrt(3.0)
    view = np.array([-1.0, 0.0, 0.0])
    h = (view + light) / np.linalg.norm(view + light)
    sh = 0.01 + max(n @ light, 0) ** 3 + max(n @ h, 0) ** 32
    assert img[32, 32, 0] == pytest.approx(sh, rel=2e-6)
    assert img[32, 32, 1] == 0.0 and img[32, 32, 2] == 0.0 and img[32, 32, 3] == 1.0
    # corners see the clear colour (window.rs:948-953)
    assert np.allclose(img[0, 0], [0.01, 0.01, 0.02, 1.0])


def test_oracle_colors_and_gradient():
    """get_color (shader.wgsl:38-64) and the speed gradient (:86-113)."""
    grad = ((0.0, 0.0, 0.0, 1.0), (0.5, 0.5, 0.5, 1.0), (1.0, 1.0, 1.0, 1.0))
    table = [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1)]
    for i in range(12):
        assert splat_ref.instance_color(0, [0, 0, 0], [1.0, 0.1, float(i)], grad, (0, 1)) == list(table[i % 6])
    c = splat_ref.instance_color(1, [0.3, 0.4, 0.0], [1, 0.1, 0], grad, (0.0, 1.0))   # |v| = 0.5
    assert [float(x) for x in c] == pytest.approx([0.5, 0.5, 0.5])
    c = splat_ref.instance_color(1, [0.15, 0.2, 0.0], [1, 0.1, 0], grad, (0.0, 1.0))  # |v| = 0.25
    assert [float(x) for x in c] == pytest.approx([0.25, 0.25, 0.25])
    c = splat_ref.instance_color(1, [9.0, 0.0, 0.0], [1, 0.1, 0], grad, (2.0, 2.0))   # empty range -> max
    assert [float(x) for x in c] == [1.0, 1.0, 1.0]


def test_oracle_box_edges():
    """bounding_box.wgsl:47-59: a pixel whose ray crosses a box edge is
    lightened (alpha 0.1 over the clear colour), a face interior is not."""
    from moldyn_gb300.render import Camera
    cam = Camera((-3.0, 0.5, 0.5), 60.0, 101, 101)
    img = splat_ref.render(np.zeros((0, 12), np.float32), _params(cam, box=[1.0, 1.0, 1.0]), 101, 101)
    bg = np.float32(0.01)
    centre = img[50, 50, 0]
    assert centre == bg                      # looking through two face interiors
    lit = img[:, :, 0] > bg
    assert lit.any() and lit.sum() < 0.2 * lit.size
    # a pixel on both the front and back silhouettes gets two blends
    assert np.isclose(img[:, :, 0].max(), np.float32(0.1) + np.float32(0.9) * (np.float32(0.1) + np.float32(0.9) * bg),
                      rtol=1e-6) or np.isclose(img[:, :, 0].max(), np.float32(0.1) + np.float32(0.9) * bg)


def test_ppm_round_trip(tmp_path):
    from moldyn_gb300.render import read_ppm, write_ppm
    img = np.random.default_rng(1).uniform(0, 1, (7, 5, 4)).astype(np.float32)
    write_ppm(str(tmp_path / "a.ppm"), img)
    back = read_ppm(str(tmp_path / "a.ppm"))
    assert back.shape == (7, 5, 3)
    assert np.array_equal(back, np.round(img[:, :, :3] * 255).astype(np.uint8))


# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("mode,seed,with_box", [(0, 1, True), (1, 2, True), (0, 3, False)])
def test_splat_matches_oracle(mode, seed, with_box):
    from moldyn_gb300 import render as rnd
    parts = _scene(seed, 70)
    cam = rnd.framing_camera([4.0, 4.0, 4.0], 96, 72)
    cam.update(cam.eye, (1.0, 0.15, -0.1), 96, 72)
    box = [4.0, 4.0, 4.0] if with_box else None
    prm = rnd.splat_params(cam, mode, speed_range=(0.2, 1.5), box=box)
    got = rnd.splat(parts, prm, 96, 72)
    want = splat_ref.render(parts, _params(cam, mode, box, grange=(0.2, 1.5)), 96, 72)
    assert got.shape == want.shape
    bad = np.argwhere(np.any(got != want, axis=2))
    assert len(bad) == 0, f"{len(bad)} pixels differ, first {bad[:5].tolist()}"
    assert (got[:, :, 0] + got[:, :, 1] + got[:, :, 2] > 0.05).sum() > 200   # spheres are on screen


@pytest.mark.gpu
def test_splat_depth_ties_and_camera_inside():
    """Equal depths: the lower instance wins (strict depth test over instances
    in order); a sphere around the camera is culled (back faces)."""
    from moldyn_gb300 import render as rnd
    cam = rnd.Camera((0.0, 0.0, 0.0), 70.0, 48, 40)
    p = np.zeros((4, 12), dtype=np.float32)
    for i in range(3):
        p[i, 0:4] = [3.0, 0.2, 0.1, 1.0]
        p[i, 9] = 0.8
        p[i, 10] = float(i + 1)        # green, blue, yellow: identical spheres
    p[3, 0:4] = [0.1, 0.0, 0.0, 1.0]   # encloses the camera
    p[3, 9] = 1.0
    p[3, 10] = 0.0
    prm = rnd.splat_params(cam, 0)
    got = rnd.splat(p, prm, 48, 40)
    want = splat_ref.render(p, _params(cam), 48, 40)
    assert np.array_equal(got, want)
    hit = got[:, :, 1] > 0.02
    assert hit.any() and not (got[:, :, 2] > 0.03).any()   # only instance 0 (green) is seen


@pytest.mark.gpu
def test_render_cli(tmp_path):
    """render: a saved frame to a PPM through the GPU path."""
    from moldyn_gb300.cli import main
    from moldyn_gb300.core import ParticleDatabase
    from moldyn_gb300.render import read_ppm
    d = str(tmp_path)
    ParticleDatabase.clear_particles()
    main(["-f", d, "initialize", "-t", "fcc", "-s", "3", "3", "3", "-n", "Argon", "-m", "66.335", "-r", "0.071",
          "-l", "0.5406", "-T", "120", "--seed", "4"])
    out = os.path.join(d, "f0.ppm")
    main(["-f", d, "render", "-s", "0", "-o", out, "--width", "160", "--height", "90", "--color-by", "speed",
          "--speed-range", "0", "2"])
    img = read_ppm(out)
    assert img.shape == (90, 160, 3)
    assert (img.astype(int).sum(axis=2) > 30).sum() > 100
