"""RGB-D camera frames (RGB888 + millimetre depth) decoded on the device with
the reference live application's conversion (scene_flow_visualization.cpp:313-323):
the solve from them equals, bit for bit, the solve of the same frames decoded
by the oracle and pushed as floats."""
import numpy as np
import pytest

from oracle import oracle
from pdflow import BatchSolver, Solver, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def camera_frames(seed, vga=False):
    """Two RGB888 + millimetre-depth frames of a seeded scene (channels spread
    around the scene's intensity so that the gray conversion is exercised)."""
    i1, z1, i2, z2 = scenes.make_pair(seed, vga=vga)
    rng = np.random.default_rng(seed)
    out = []
    for i, z in ((i1, z1), (i2, z2)):
        d = rng.integers(-12, 13, size=i.shape)
        rgb = np.stack([np.clip(i.astype(int) + d, 0, 255), i, np.clip(i.astype(int) - d, 0, 255)], axis=-1)
        out.append((rgb.astype(np.uint8), (z // 5).astype(np.uint16)))
    return out


def flow_of(s):
    return s.dxp.copy(), s.dyp.copy(), s.dzp.copy()


@pytest.mark.parametrize("rotate", [False, True])
def test_rgb_frames_solve_as_the_oracle_decode(rotate):
    frames = camera_frames(70 + int(rotate))
    a = Solver(240, 320, 240).initializeCUDA()
    for rgb, mm in frames:
        a.push_rgb(rgb, mm, rotate180=rotate)
    a.solveSceneFlowGPU()
    b = Solver(240, 320, 240).initializeCUDA()
    for rgb, mm in frames:
        I, Z = oracle.decode_frame_rgb8_mm(rgb, mm, rotate)
        b.createImagePyramidGPU(I, Z)
    b.solveSceneFlowGPU()
    for x, y in zip(flow_of(a), flow_of(b)):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    assert np.abs(a.dxp).max() > 0
    a.freeGPUMemory()
    b.freeGPUMemory()


def test_rgb_batch_equals_single_pairs():
    pairs = [camera_frames(80 + k) for k in range(3)]
    bs = BatchSolver(120, 320, 240, 3)
    for f in range(2):
        bs.push_rgb(np.stack([p[f][0] for p in pairs]), np.stack([p[f][1] for p in pairs]), rotate180=True)
    bs.solve(3)
    got = bs.read_flow(3)
    bs.close()
    for k, p in enumerate(pairs):
        s = Solver(120, 320, 240).initializeCUDA()
        for rgb, mm in p:
            s.push_rgb(rgb, mm, rotate180=True)
        s.solveSceneFlowGPU()
        for x, y in zip(flow_of(s), (g[k] for g in got)):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
        s.freeGPUMemory()
