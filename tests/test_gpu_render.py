"""The GPU scene renderer against the numpy renderer and ground truth."""
import numpy as np
import pytest

from pdflow import datagen, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("vga,seed,nobj", [(False, 3, 3), (True, 8, 6), (False, 44, 8)])
def test_noiseless_frames_and_flow_match_numpy(built_lib, vga, seed, nobj):
    torch = pytest.importorskip("torch")
    sc = scenes.make_scene(seed, vga, nobj)
    inten, depth, flow = datagen.render_scenes(torch, [sc], 0, with_flow=True, sensor_noise=False)
    z, tex = scenes._render_depth_tex(sc, 0)
    ref_d = np.clip(np.rint(z * 5000.0), 0, 65535).astype(np.int64)
    ref_i = np.clip(np.rint(tex * 255.0), 0, 255).astype(np.int64)
    got_d = depth[0].cpu().numpy().view(np.uint16).astype(np.int64)
    got_i = inten[0].cpu().numpy().astype(np.int64)
    for got, ref in ((got_d, ref_d), (got_i, ref_i)):
        diff = np.abs(got - ref)
        assert diff.max() <= 1 and (diff == 0).mean() >= 0.999
    gt = scenes.ground_truth_flow(sc, 0)
    assert np.allclose(flow[0].cpu().numpy(), gt, atol=1e-6)


def test_sensor_noise_statistics(built_lib):
    torch = pytest.importorskip("torch")
    sc = scenes.make_scene(5, vga=True)
    _, depth, _ = datagen.render_scenes(torch, [sc], 0)
    d = depth[0].cpu().numpy().view(np.uint16).astype(np.float64) / 5000.0
    z, _ = scenes._render_depth_tex(sc, 0)
    holes = d == 0
    assert 0.015 < holes.mean() < 0.025
    r = (d - z)[~holes] / (1.5e-3 * z[~holes] ** 2)
    assert abs(r.mean()) < 0.05 and 0.9 < r.std() < 1.1
