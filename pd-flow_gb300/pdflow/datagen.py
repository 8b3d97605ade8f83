"""Seeded synthetic pairs rendered on the GPU (pdflow_render_frames).

Training the warm-start network, the serving simulation and the accuracy
evaluations need many frames; the numpy renderer of `scenes` is the
specification, this module renders the same scenes on the device.  torch
only holds the device buffers.
"""
from __future__ import annotations

from . import scenes
from ._lib import render_frames


def render_scenes(torch, scene_list, k: int, with_flow: bool = False, sensor_noise: bool = True):
    """Frame k of each scene: (intensity uint8 [n,h,w], depth int16 [n,h,w] holding
    uint16 bits, ground-truth flow [n,3,w*h] float32 or None), on cuda."""
    n = len(scene_list)
    w, h = scene_list[0].width, scene_list[0].height
    inten = torch.empty((n, h, w), dtype=torch.uint8, device="cuda")
    depth = torch.empty((n, h, w), dtype=torch.int16, device="cuda")
    flow = torch.empty((n, 3, w * h), dtype=torch.float32, device="cuda") if with_flow else None
    descs = [scenes.frame_desc(sc, k, sensor_noise) for sc in scene_list]
    render_frames(descs, inten.data_ptr(), depth.data_ptr(), flow.data_ptr() if with_flow else None,
                  torch.cuda.current_stream().cuda_stream)
    return inten, depth, flow


def render_pairs(torch, seeds, vga: bool, n_objects=None, with_flow: bool = False):
    """(I1, Z1, I2, Z2[, flow]) for seeds: frames 0 and 1 of scenes.make_scene(seed).
    n_objects: None (default count), an int, or a function of the seed."""
    scs = []
    for s in seeds:
        nobj = n_objects(s) if callable(n_objects) else n_objects
        scs.append(scenes.make_scene(int(s), vga, nobj))
    i1, z1, gt = render_scenes(torch, scs, 0, with_flow)
    i2, z2, _ = render_scenes(torch, scs, 1)
    return (i1, z1, i2, z2, gt) if with_flow else (i1, z1, i2, z2)
