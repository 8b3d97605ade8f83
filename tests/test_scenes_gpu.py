"""The torch scene renderer (training data) against the numpy renderer."""
import numpy as np
import pytest

from pdflow import scenes, scenes_gpu


@pytest.mark.parametrize("seed,n_obj", [(3, 3), (8, 6)])
def test_noiseless_render_matches_numpy(seed, n_obj):
    torch = pytest.importorskip("torch")
    sc = scenes.make_scene(seed, vga=False, n_objects=n_obj)
    for k in (0, 1):
        z_ref, t_ref = scenes._render_depth_tex(sc, k)
        z, t = scenes_gpu.render_depth_tex(torch, sc, k, "cpu")
        assert np.allclose(z.numpy(), z_ref, rtol=1e-12, atol=1e-12)
        assert np.allclose(t.numpy(), t_ref, rtol=1e-12, atol=1e-12)


def test_noisy_render_statistics():
    torch = pytest.importorskip("torch")
    sc = scenes.make_scene(5, vga=False)
    i, z = scenes_gpu.render(torch, sc, 0, "cpu")
    zu = z.numpy().view(np.uint16)
    assert i.dtype == torch.uint8 and zu.shape == (240, 320)
    holes = (zu == 0).mean()
    assert 0.01 < holes < 0.03
    z_ref, _ = scenes._render_depth_tex(sc, 0)
    valid = zu > 0
    assert np.abs(zu[valid] / 5000.0 - z_ref[valid]).mean() < 0.02
