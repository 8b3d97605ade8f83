"""Batch renderer of the seeded synthetic scenes on a torch device.

Training the warm-start network needs tens of thousands of labelled pairs;
the numpy renderer of `scenes` takes about a second per VGA frame, so this
module renders the same scenes (geometry, motions and textures from
`scenes.make_scene`, float64 ray casting with the same formulas) with torch
on the GPU.  Only the per-frame sensor noise differs: depth noise and holes
come from a torch generator seeded from the scene, not from numpy's.
"""
from __future__ import annotations

import numpy as np

from . import scenes


def _noise(torch, tex, pts):
    """scenes._Noise3 evaluated on pts [N, 3] (float64 tensor)."""
    dev = pts.device
    perm = torch.as_tensor(tex.perm, device=dev)
    vals = torch.as_tensor(tex.vals, device=dev)

    def octave(q_pts, scale):
        q = q_pts / (tex.cell * scale)
        f = torch.floor(q)
        t = q - f
        t = t * t * (3.0 - 2.0 * t)
        i = f.to(torch.int64)
        out = torch.zeros(q.shape[0], dtype=torch.float64, device=dev)
        for dx in (0, 1):
            wx = t[:, 0] if dx else 1.0 - t[:, 0]
            for dy in (0, 1):
                wy = t[:, 1] if dy else 1.0 - t[:, 1]
                for dz in (0, 1):
                    wz = t[:, 2] if dz else 1.0 - t[:, 2]
                    ix, iy, iz = i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz
                    lat = vals[perm[(perm[(perm[ix & 255] + iy) & 255] + iz) & 255]]
                    out = out + wx * wy * wz * lat
        return out

    return 0.65 * octave(pts, 1.0) + 0.35 * octave(pts + 17.0, 0.5)


def render_depth_tex(torch, scene: scenes.Scene, k: int, device):
    """(z, tex) [h, w] float64 tensors of frame k (scenes._render_depth_tex)."""
    cam = scene.cam
    w, h = cam["width"], cam["height"]
    vv, uu = torch.meshgrid(torch.arange(h, dtype=torch.float64, device=device),
                            torch.arange(w, dtype=torch.float64, device=device), indexing="ij")
    xn = ((uu - cam["cx"]) / cam["fx"]).reshape(-1)
    yn = ((vv - cam["cy"]) / cam["fy"]).reshape(-1)
    d = torch.stack([xn, yn, torch.ones_like(xn)], dim=1)
    z0, a, b = scene.plane
    zbest = z0 / (1.0 - a * xn - b * yn)
    tex = 0.15 + 0.8 * _noise(torch, scene.plane_tex, d * zbest[:, None])
    inf = torch.full_like(xn, float("inf"))
    for ob in scene.objects:
        c_np, r_np = ob.pose(k)
        c = torch.as_tensor(c_np, device=device)
        r = torch.as_tensor(r_np, device=device)
        if ob.kind == "sphere":
            rad = float(ob.size[0])
            dd = (d * d).sum(dim=1)
            dc = d @ c
            disc = dc * dc - dd * (float(c_np @ c_np) - rad * rad)
            hit = disc > 0
            t = torch.where(hit, (dc - torch.sqrt(torch.clamp(disc, min=0.0))) / dd, inf)
        else:
            o_l = r.T @ (-c)
            d_l = d @ r
            size = torch.as_tensor(ob.size, device=device)
            inv = 1.0 / d_l
            t1 = (-size[None, :] - o_l[None, :]) * inv
            t2 = (size[None, :] - o_l[None, :]) * inv
            tn = torch.nan_to_num(torch.minimum(t1, t2), nan=-float("inf")).amax(dim=1)
            tf = torch.nan_to_num(torch.maximum(t1, t2), nan=float("inf")).amin(dim=1)
            hit = (tn <= tf) & (tf > 0)
            t = torch.where(hit, tn, inf)
        closer = t < zbest
        if bool(closer.any()):
            zbest = torch.where(closer, t, zbest)
            idx = torch.nonzero(closer).squeeze(1)
            p_local = (d[idx] * t[idx, None] - c[None, :]) @ r
            tex[idx] = ob.albedo * (0.1 + 0.9 * _noise(torch, ob.tex, p_local))
    return zbest.reshape(h, w), tex.reshape(h, w)


def render(torch, scene: scenes.Scene, k: int, device, noise: bool = True):
    """(intensity uint8, depth int16 holding uint16 bits) [h, w] tensors of frame k."""
    z, tex = render_depth_tex(torch, scene, k, device)
    if noise:
        g = torch.Generator(device=device)
        g.manual_seed(int(scene.noise_seed) * 1009 + k)
        z = z + torch.randn(z.shape, generator=g, dtype=torch.float64, device=device) * (1.5e-3 * z * z)
        holes = torch.rand(z.shape, generator=g, dtype=torch.float64, device=device) < 0.02
    depth = torch.clamp(torch.round(z * 5000.0), 0, 65535).to(torch.int32)
    if noise:
        depth = torch.where(holes, torch.zeros_like(depth), depth)
    inten = torch.clamp(torch.round(tex * 255.0), 0, 255).to(torch.uint8)
    return inten, (depth - 65536 * (depth >= 32768).to(torch.int32)).to(torch.int16)


def make_pairs(torch, seeds, vga: bool, device, n_objects=None):
    """Stacks (I1, Z1, I2, Z2), each [len(seeds), h, w] (uint8 / int16 bits of uint16)."""
    out = [[], [], [], []]
    for s in seeds:
        nobj = n_objects(s) if callable(n_objects) else n_objects
        sc = scenes.make_scene(int(s), vga, nobj)
        i1, z1 = render(torch, sc, 0, device)
        i2, z2 = render(torch, sc, 1, device)
        for lst, t in zip(out, (i1, z1, i2, z2)):
            lst.append(t)
    return [torch.stack(x) for x in out]


def as_numpy_u16(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint16)
