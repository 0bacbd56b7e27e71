"""CPU restatement of the GUI viewer's render pass -- test infrastructure.

The oracle for moldyn_gb300/csrc/splat.cu (mdgb_splat); only the tests use it.
It restates, with IEEE float32 numpy operations in the kernel's order:

* gui/src/visualizer/shader.wgsl:38-64 get_color (id % 6), :86-113 the speed
  gradient (mix(a, b, w) = a (1 - w) + b w), :121-130 the fragment shading
  0.01 + max(n.l, 0)^3 + max(n.h, 0)^32, l = -normalize(1, -1, 1);
* gui/src/visualizer/bounding_box.wgsl:47-59 the edge mask (two of three local
  coordinates with |p - 1/2| > 0.495), blended at alpha 0.1 (wgpu
  ALPHA_BLENDING, window.rs:665) on the box faces in front of the nearest
  particle (depth test "less", no depth write, window.rs:650-651);
* window.rs:940-990 the frame: clear colour (0.01, 0.01, 0.02, 1), particles
  with depth test "less" in instance order (the lower index wins on equal
  depth), back faces culled.

Spheres are exact (ray-cast), as in the kernel; the GUI's 92-vertex icosphere
would show facets.  Every pixel is tested against every particle (no screen
boxes), so the kernel's culling is checked too.  pow(x, 3) = x*x*x,
pow(x, 32) = five squarings, normalize(v) = v / sqrt(v.v): the WGSL built-ins
are implementation-defined, these are the exact forms the kernel uses.
"""
from __future__ import annotations

import numpy as np

F = np.float32


def _dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def pixel_rays(view, p00, p11, width, height):
    """(3, H, W) world-space ray directions through pixel centres."""
    px = np.arange(width, dtype=F)[None, :]
    py = np.arange(height, dtype=F)[:, None]
    xn = ((px + F(0.5)) / F(width)) * F(2.0) - F(1.0)
    yn = F(1.0) - ((py + F(0.5)) / F(height)) * F(2.0)
    vx = np.broadcast_to(xn / F(p00), (height, width))
    vy = np.broadcast_to(yn / F(p11), (height, width))
    return np.stack([(F(view[j * 4 + 0]) * vx + F(view[j * 4 + 1]) * vy) - F(view[j * 4 + 2]) for j in range(3)])


def hit_t(eye, d, c, r, znear, zfar):
    """Nearest front intersection parameter (view depth) or inf."""
    oc = [F(c[k]) - F(eye[k]) for k in range(3)]
    b = _dot(d, oc)
    a = _dot(d, d)
    cc = ((oc[0] * oc[0] + oc[1] * oc[1]) + oc[2] * oc[2]) - F(r) * F(r)
    disc = b * b - a * cc
    with np.errstate(invalid="ignore"):
        t = (b - np.sqrt(disc)) / a
    ok = (disc >= 0) & (t >= znear) & (t <= zfar)
    return np.where(ok, t, F(np.inf)).astype(F)


def _normalize(v):
    l = np.sqrt(_dot(v, v))
    return [v[0] / l, v[1] / l, v[2] / l]


def instance_color(mode, vel, mri, grad, grange):
    if mode == 0:
        table = [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1)]
        return [F(x) for x in table[int(np.uint32(F(mri[2]))) % 6]]
    if mode == 1:
        gm, gM = F(grange[0]), F(grange[1])
        v3 = [F(vel[0]), F(vel[1]), F(vel[2])]
        v = (np.sqrt(_dot(v3, v3)) - gm) / (gM - gm) if gM != gm else F(1.0)
        if gM <= gm:
            v = F(1.0)
        lo, hi = (grad[0], grad[1]) if v < F(0.5) else (grad[1], grad[2])
        w = v * F(2.0) if v < F(0.5) else (v - F(0.5)) * F(2.0)
        return [F(lo[k]) * (F(1.0) - w) + F(hi[k]) * w for k in range(3)]
    return [F(0.0)] * 3


def render(particles, params: dict, width: int, height: int) -> np.ndarray:
    """particles: (n, 12) float32 (ParticleDataLite); params: view_pos, view,
    proj, gradient (3 colours), grange (min, max), mode, box (or None)."""
    parts = np.asarray(particles, dtype=F).reshape(-1, 12)
    eye = np.asarray(params["view_pos"], dtype=F)[:3]
    view = np.asarray(params["view"], dtype=F)
    proj = np.asarray(params["proj"], dtype=F)
    a, b = F(proj[10]), F(proj[14])
    znear, zfar = b / (a - F(1.0)), b / (a + F(1.0))
    d = pixel_rays(view, proj[0], proj[5], width, height)
    best_t = np.full((height, width), np.inf, dtype=F)
    best_i = np.full((height, width), -1, dtype=np.int64)
    for i in range(parts.shape[0]):
        t = hit_t(eye, d, parts[i, 0:3], parts[i, 9], znear, zfar)
        better = t < best_t            # strict: the lower index keeps equal depths
        best_t = np.where(better, t, best_t)
        best_i = np.where(better, i, best_i)
    img = np.zeros((height, width, 4), dtype=F)
    img[:, :, 0], img[:, :, 1], img[:, :, 2], img[:, :, 3] = F(0.01), F(0.01), F(0.02), F(1.0)
    light = _normalize([F(1.0), F(-1.0), F(1.0)])
    light = [-light[0], -light[1], -light[2]]
    grad = params.get("gradient")
    grange = params.get("grange", (0.0, 1.0))
    for y, x in zip(*np.nonzero(best_i >= 0)):
        i = best_i[y, x]
        c = parts[i, 0:3]
        r = F(parts[i, 9])
        t = best_t[y, x]
        dd = d[:, y, x]
        nrm = _normalize([(eye[k] + t * dd[k]) - c[k] for k in range(3)])
        pos = [c[k] + nrm[k] * r for k in range(3)]
        vv = _normalize([eye[k] - pos[k] for k in range(3)])
        h = _normalize([vv[k] + light[k] for k in range(3)])
        dl = max(_dot(nrm, light), F(0.0))
        dh = max(_dot(nrm, h), F(0.0))
        p3 = (dl * dl) * dl
        for _ in range(5):
            dh = dh * dh
        sh = (F(0.01) + p3) + dh
        col = instance_color(params["mode"], parts[i, 4:7], parts[i, 8:11], grad, grange)
        img[y, x, 0:3] = [col[k] * sh for k in range(3)]
    box = params.get("box")
    if box is not None:
        box = [F(v) for v in box[:3]]
        ok = np.ones((height, width), dtype=bool)
        te = np.full((height, width), -1e30, dtype=F)
        tx = np.full((height, width), 1e30, dtype=F)
        for k in range(3):
            zero = d[k] == 0
            ok &= ~(zero & ((eye[k] < 0) | (eye[k] > box[k])))
            with np.errstate(divide="ignore", invalid="ignore"):
                ta = (F(0.0) - eye[k]) / d[k]
                tb = (box[k] - eye[k]) / d[k]
            te = np.where(zero, te, np.maximum(te, np.minimum(ta, tb)))
            tx = np.where(zero, tx, np.minimum(tx, np.maximum(ta, tb)))
        tz = np.where(best_i >= 0, best_t, zfar)
        for tf in (te, tx):
            sel = ok & (te <= tx) & (tf >= znear) & (tf < tz)
            edges = []
            for k in range(3):
                l = (eye[k] + tf * d[k]) / box[k]
                edges.append(np.abs(l - F(0.5)) > F(0.495))
            edge = (edges[0] & edges[1]) | (edges[0] & edges[2]) | (edges[1] & edges[2])
            sel &= edge
            for k in range(3):
                img[:, :, k] = np.where(sel, F(0.1) + F(0.9) * img[:, :, k], img[:, :, k])
    return img
