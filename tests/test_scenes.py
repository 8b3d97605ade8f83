"""The seeded synthetic RGB-D generator produces the workloads' statistics."""
import numpy as np
import pytest

from pdflow import scenes


@pytest.mark.parametrize("vga", [False, True])
def test_pair_shapes_and_ranges(vga):
    i1, z1, i2, z2 = scenes.make_pair(3, vga=vga)
    h, w = (480, 640) if vga else (240, 320)
    for a, dt in ((i1, np.uint8), (i2, np.uint8), (z1, np.uint16), (z2, np.uint16)):
        assert a.shape == (h, w) and a.dtype == dt
    for z in (z1, z2):
        valid = z[z > 0] / 5000.0
        assert 0.7 < valid.min() and valid.max() < 4.3           # objects 0.8-2.5 m, plane 2-4 m, noise
        holes = float(np.mean(z == 0))
        assert 0.01 < holes < 0.03                               # 2 % holes
    assert i1.std() > 10                                         # textured


def test_deterministic_per_seed():
    a = scenes.make_pair(7)
    b = scenes.make_pair(7)
    c = scenes.make_pair(8)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert not np.array_equal(a[1], c[1])


def test_object_motion_is_bounded():
    sc = scenes.make_scene(5, vga=True, n_objects=8)
    for ob in sc.objects:
        assert np.linalg.norm(ob.d_center) <= 0.05 + 1e-12
        ang = np.degrees(np.arccos(np.clip((np.trace(ob.d_rot) - 1) / 2, -1, 1)))
        assert ang <= 3.0 + 1e-9
        assert 0.8 <= ob.center[2] <= 2.5


def test_frames_differ_only_where_objects_move():
    i1, z1, i2, z2 = scenes.make_pair(4, n_objects=2)
    both = (z1 > 0) & (z2 > 0)
    dz = np.abs(z1.astype(np.int64) - z2.astype(np.int64))[both] / 5000.0
    assert np.median(dz) < 0.02                                  # static plane: only noise
    assert np.mean(i1 != i2) > 0.001                             # something moved


def test_decode_matches_reference_packing():
    i1, z1, _, _ = scenes.make_pair(1)
    I, Z = scenes.decode(i1, z1)
    h, w = i1.shape
    assert I[5 + 7 * h] == i1[5, 7]
    assert Z[5 + 7 * h] == np.float32(z1[5, 7]) * np.float32(1 / 5000)


def test_ground_truth_flow_is_zero_on_the_plane_and_bounded_on_objects():
    sc = scenes.make_scene(12, vga=False, n_objects=4)
    gt = scenes.ground_truth_flow(sc, 0)
    assert gt.shape == (3, 320 * 240)
    mag = np.sqrt((gt ** 2).sum(axis=0))
    moving = mag > 0
    assert 0.01 < moving.mean() < 0.9          # objects cover part of the image, the plane is static
    assert mag.max() < 0.05 + 3 * np.pi / 180 * 0.4   # <= 5 cm translation + 3 deg about a centre <= 0.4 m away


def test_ground_truth_flow_of_a_translating_object_is_its_translation():
    sc = scenes.make_scene(21, vga=False, n_objects=1)
    ob = sc.objects[0]
    ob.d_rot = np.eye(3)                      # pure translation
    gt = scenes.ground_truth_flow(sc, 0)
    moving = np.sqrt((gt ** 2).sum(axis=0)) > 0
    dx, dy, dz = ob.d_center[2], ob.d_center[0], ob.d_center[1]   # depth, horizontal, vertical
    assert np.allclose(gt[0][moving], dx) and np.allclose(gt[1][moving], dy) and np.allclose(gt[2][moving], dz)
