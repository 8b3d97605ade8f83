"""Seeded synthetic RGB-D scenes for the solver's workloads.

The reference ships no data, so every workload is rendered here from a seed:
a textured plane at 2-4 m plus boxes and spheres at 0.8-2.5 m, each object
moving rigidly by at most 5 cm and 3 degrees between the two frames.

* intensity: uint8 smoothed value noise (0-255) fixed to each surface, so the
  texture moves with its object;
* depth: uint16 = z * 5000 (the reference's PNG depth scale,
  scene_flow_impair.cpp:242), Gaussian noise sigma = 1.5e-3 * z^2 and 2 %
  zero holes, drawn independently per frame;
* cameras: QVGA 320x240, fx = fy = 262.5, c = (160, 120); VGA 640x480,
  fx = fy = 525, c = (320, 240).

Images are row-major (height, width), as a PNG decoder returns them.
Streams (for the serving loop) keep each object's per-frame rigid motion, so
frame k is the scene after k steps of a constant-velocity trajectory, or, with
`period`, of a trajectory that reverses every `period` frames and so stays in
view for any number of frames.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

QVGA = dict(width=320, height=240, fx=262.5, fy=262.5, cx=160.0, cy=120.0)
VGA = dict(width=640, height=480, fx=525.0, fy=525.0, cx=320.0, cy=240.0)


def _rotation(axis: np.ndarray, angle: float) -> np.ndarray:
    axis = axis / np.linalg.norm(axis)
    x, y, z = axis
    c, s = math.cos(angle), math.sin(angle)
    C = 1.0 - c
    return np.array([[c + x * x * C, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, c + y * y * C, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, c + z * z * C]])


class _Noise3:
    """Two-octave 3D value noise on an integer lattice (hash-table based)."""

    def __init__(self, rng: np.random.Generator, cell: float):
        self.perm = rng.permutation(256).astype(np.int64)
        self.vals = rng.random(256)
        self.cell = cell

    def _lattice(self, ix, iy, iz):
        p = self.perm
        return self.vals[p[(p[(p[ix & 255] + iy) & 255] + iz) & 255]]

    def _octave(self, pts: np.ndarray, scale: float) -> np.ndarray:
        q = pts / (self.cell * scale)
        f = np.floor(q)
        t = q - f
        t = t * t * (3.0 - 2.0 * t)
        i = f.astype(np.int64)
        out = 0.0
        for dx in (0, 1):
            wx = t[:, 0] if dx else 1.0 - t[:, 0]
            for dy in (0, 1):
                wy = t[:, 1] if dy else 1.0 - t[:, 1]
                for dz in (0, 1):
                    wz = t[:, 2] if dz else 1.0 - t[:, 2]
                    out = out + wx * wy * wz * self._lattice(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
        return out

    def __call__(self, pts: np.ndarray) -> np.ndarray:
        return (0.65 * self._octave(pts, 1.0) + 0.35 * self._octave(pts + 17.0, 0.5)) / 1.0


@dataclasses.dataclass
class _Object:
    kind: str               # "sphere" | "box"
    center: np.ndarray      # (3,) camera frame, metres
    rot: np.ndarray         # (3,3) object -> camera
    size: np.ndarray        # sphere: (r,), box: half extents (3,)
    tex: _Noise3
    d_center: np.ndarray    # per-frame translation
    d_rot: np.ndarray       # per-frame rotation (about the object's centre)
    albedo: float
    period: int = 0         # > 0: the motion reverses every `period` frames (bounded trajectory)

    def pose(self, k: int):
        steps = k
        if self.period > 0:   # triangle wave: forward `period` frames, back `period` frames
            m = k % (2 * self.period)
            steps = m if m <= self.period else 2 * self.period - m
        c, r = self.center.copy(), self.rot.copy()
        for _ in range(steps):
            c = c + self.d_center
            r = self.d_rot @ r
        return c, r


@dataclasses.dataclass
class Scene:
    cam: dict
    plane: tuple            # (z0, a, b): z = z0 + a*x + b*y
    plane_tex: _Noise3
    objects: list
    noise_seed: int

    @property
    def width(self):
        return self.cam["width"]

    @property
    def height(self):
        return self.cam["height"]


def make_scene(seed: int, vga: bool = False, n_objects: int | None = None, period: int = 0) -> Scene:
    """Scene for `seed`: plane at 2-4 m plus `n_objects` boxes/spheres at 0.8-2.5 m
    (default 6 at VGA, 3 at QVGA), each with a rigid motion of <= 5 cm and <= 3 deg
    per frame.  period > 0 makes long sequences stay in view: each object moves
    forward for `period` frames, then back (frames 0 and 1 do not depend on it)."""
    rng = np.random.default_rng(seed)
    cam = dict(VGA if vga else QVGA)
    if n_objects is None:
        n_objects = 6 if vga else 3
    # plane z = z0 + a x + b y, kept inside [2, 4] m over the field of view
    xmax = cam["cx"] / cam["fx"]
    ymax = cam["cy"] / cam["fy"]
    while True:
        z0 = rng.uniform(2.6, 3.4)
        a, b = rng.uniform(-0.35, 0.35, size=2)
        corners = [z0 / (1.0 - a * sx * xmax - b * sy * ymax) for sx in (-1, 1) for sy in (-1, 1)]
        if min(corners) >= 2.0 and max(corners) <= 4.0 and min(1.0 - abs(a) * xmax - abs(b) * ymax, 1) > 0:
            break
    plane_tex = _Noise3(rng, 0.04)
    objs = []
    for _ in range(n_objects):
        kind = "sphere" if rng.random() < 0.5 else "box"
        zc = rng.uniform(1.0, 2.3)
        xc = rng.uniform(-0.7, 0.7) * xmax * zc
        yc = rng.uniform(-0.7, 0.7) * ymax * zc
        if kind == "sphere":
            size = np.array([rng.uniform(0.08, min(0.22, zc - 0.8))])
        else:
            size = rng.uniform(0.06, min(0.18, zc - 0.8), size=3)
        rot = _rotation(rng.normal(size=3), rng.uniform(0, math.pi))
        tdir = rng.normal(size=3)
        d_center = tdir / np.linalg.norm(tdir) * rng.uniform(0.01, 0.05)
        d_rot = _rotation(rng.normal(size=3), math.radians(rng.uniform(0.5, 3.0)))
        objs.append(_Object(kind, np.array([xc, yc, zc]), rot, size, _Noise3(rng, rng.uniform(0.015, 0.04)),
                            d_center, d_rot, rng.uniform(0.6, 1.0), period))
    return Scene(cam, (z0, a, b), plane_tex, objs, int(rng.integers(1 << 31)))


def _render_depth_tex(scene: Scene, k: int):
    cam = scene.cam
    w, h = cam["width"], cam["height"]
    uu, vv = np.meshgrid(np.arange(w, dtype=np.float64), np.arange(h, dtype=np.float64))
    xn = ((uu - cam["cx"]) / cam["fx"]).ravel()
    yn = ((vv - cam["cy"]) / cam["fy"]).ravel()
    d = np.stack([xn, yn, np.ones_like(xn)], axis=1)          # ray direction, t = depth
    z0, a, b = scene.plane
    zbest = z0 / (1.0 - a * xn - b * yn)
    pts = d * zbest[:, None]
    tex = 0.15 + 0.8 * scene.plane_tex(pts)
    for ob in scene.objects:
        c, r = ob.pose(k)
        if ob.kind == "sphere":
            rad = ob.size[0]
            dd = np.einsum("ij,ij->i", d, d)
            dc = d @ c
            disc = dc * dc - dd * (c @ c - rad * rad)
            hit = disc > 0
            t = np.full_like(xn, np.inf)
            t[hit] = (dc[hit] - np.sqrt(disc[hit])) / dd[hit]
        else:
            o_l = r.T @ (-c)                                   # ray origin in box frame
            d_l = d @ r                                        # == (r.T @ d.T).T
            with np.errstate(divide="ignore", invalid="ignore"):
                inv = 1.0 / d_l
                t1 = (-ob.size[None, :] - o_l[None, :]) * inv
                t2 = (ob.size[None, :] - o_l[None, :]) * inv
            tn = np.nanmax(np.minimum(t1, t2), axis=1)
            tf = np.nanmin(np.maximum(t1, t2), axis=1)
            hit = (tn <= tf) & (tf > 0)
            t = np.where(hit, tn, np.inf)
        closer = t < zbest
        if np.any(closer):
            zbest = np.where(closer, t, zbest)
            p_local = (d[closer] * t[closer, None] - c[None, :]) @ r
            tex[closer] = ob.albedo * (0.1 + 0.9 * ob.tex(p_local))
    return zbest.reshape(h, w), tex.reshape(h, w)


def render(scene: Scene, k: int):
    """Frame k of `scene`: (intensity uint8 [h,w], depth uint16 [h,w]), row-major."""
    z, tex = _render_depth_tex(scene, k)
    rng = np.random.default_rng([scene.noise_seed, k])
    zn = z + rng.normal(size=z.shape) * (1.5e-3 * z * z)
    holes = rng.random(z.shape) < 0.02
    depth = np.clip(np.rint(zn * 5000.0), 0, 65535).astype(np.uint16)
    depth[holes] = 0
    inten = np.clip(np.rint(tex * 255.0), 0, 255).astype(np.uint8)
    return inten, depth


def _tex_desc(tex: _Noise3):
    from ._lib import NoiseTex
    t = NoiseTex()
    t.perm[:] = [int(x) for x in tex.perm]
    t.vals[:] = [float(x) for x in tex.vals]
    t.cell = float(tex.cell)
    return t


def frame_desc(scene: Scene, k: int, sensor_noise: bool = True):
    """The GPU renderer's descriptor (pdflow_scene_frame) of frame k: the same
    geometry and textures as `render`; the sensor noise comes from the
    renderer's counter-based generator keyed by (noise_seed, k)."""
    from ._lib import SceneFrame, SceneObject
    f = SceneFrame()
    cam = scene.cam
    f.width, f.height = cam["width"], cam["height"]
    f.fx, f.fy, f.cx, f.cy = cam["fx"], cam["fy"], cam["cx"], cam["cy"]
    f.plane[:] = list(scene.plane)
    f.plane_tex = _tex_desc(scene.plane_tex)
    f.n_objects = len(scene.objects)
    f.sensor_noise = 1 if sensor_noise else 0
    f.noise_seed = (int(scene.noise_seed) * 1_000_003 + k) & 0xFFFFFFFFFFFFFFFF
    for j, ob in enumerate(scene.objects):
        o = SceneObject()
        o.kind = 0 if ob.kind == "sphere" else 1
        c, r = ob.pose(k)
        cn, rn = ob.pose(k + 1)
        o.center[:] = list(c)
        o.rot[:] = list(r.ravel())
        o.next_center[:] = list(cn)
        o.next_rot[:] = list(rn.ravel())
        sz = list(ob.size) + [0.0] * (3 - len(ob.size))
        o.size[:] = sz
        o.albedo = float(ob.albedo)
        o.tex = _tex_desc(ob.tex)
        f.objects[j] = o
    return f


def ground_truth_flow(scene: Scene, k: int) -> np.ndarray:
    """Motion of each pixel's surface point from frame k to k+1, [3, w*h],
    in the solver's output convention: dx = depth change, dy = horizontal,
    dz = vertical (metres), column-major (idx = v + u * height)."""
    cam = scene.cam
    w, h = cam["width"], cam["height"]
    uu, vv = np.meshgrid(np.arange(w, dtype=np.float64), np.arange(h, dtype=np.float64))
    xn = ((uu - cam["cx"]) / cam["fx"]).ravel()
    yn = ((vv - cam["cy"]) / cam["fy"]).ravel()
    d = np.stack([xn, yn, np.ones_like(xn)], axis=1)
    z0, a, b = scene.plane
    zbest = z0 / (1.0 - a * xn - b * yn)
    hit = np.full(xn.shape, -1)
    for j, ob in enumerate(scene.objects):
        c, r = ob.pose(k)
        if ob.kind == "sphere":
            rad = ob.size[0]
            dd = np.einsum("ij,ij->i", d, d)
            dc = d @ c
            disc = dc * dc - dd * (c @ c - rad * rad)
            t = np.full_like(xn, np.inf)
            ok = disc > 0
            t[ok] = (dc[ok] - np.sqrt(disc[ok])) / dd[ok]
        else:
            o_l = r.T @ (-c)
            d_l = d @ r
            with np.errstate(divide="ignore", invalid="ignore"):
                inv = 1.0 / d_l
                t1 = (-ob.size[None, :] - o_l[None, :]) * inv
                t2 = (ob.size[None, :] - o_l[None, :]) * inv
            tn = np.nanmax(np.minimum(t1, t2), axis=1)
            tf = np.nanmin(np.maximum(t1, t2), axis=1)
            t = np.where((tn <= tf) & (tf > 0), tn, np.inf)
        closer = t < zbest
        zbest = np.where(closer, t, zbest)
        hit = np.where(closer, j, hit)
    P = d * zbest[:, None]
    gt = np.zeros_like(P)
    for j, ob in enumerate(scene.objects):
        m = hit == j
        if not m.any():
            continue
        c, r = ob.pose(k)
        cn, rn = ob.pose(k + 1)
        L = (P[m] - c[None, :]) @ r
        gt[m] = L @ rn.T + cn[None, :] - P[m]
    gt = gt.reshape(h, w, 3).transpose(1, 0, 2).reshape(-1, 3)     # column-major
    return np.stack([gt[:, 2], gt[:, 0], gt[:, 1]])


def make_pair(seed: int, vga: bool = False, n_objects: int | None = None):
    """(I1, Z1, I2, Z2) for `seed`: uint8/uint16 row-major images of frames 0 and 1."""
    sc = make_scene(seed, vga, n_objects)
    i1, z1 = render(sc, 0)
    i2, z2 = render(sc, 1)
    return i1, z1, i2, z2


def decode(intensity: np.ndarray, depth: np.ndarray):
    """Host decode to the reference's float staging buffers: column-major
    (idx = v + u*height), I = float(uint8), Z = uint16 * float32(1/5000)
    (scene_flow_impair.cpp:230-245)."""
    scale = np.float32(1.0 / 5000.0)
    I = np.ascontiguousarray(intensity.T).astype(np.float32).ravel()
    Z = (np.ascontiguousarray(depth.T).astype(np.float32) * scale).astype(np.float32).ravel()
    return I, Z
