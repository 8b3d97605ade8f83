"""The per-level record: copyAllSolutions after every level, as the reference's
live application calls it while the solve climbs the pyramid
(scene_flow_visualization.cpp:194-199; pdflow_cudalib.cu:224-237).

Every level's median-filtered image-plane flow equals the reference's own
du_l, dv_l, dw_l of that level (golden vectors of the rows = 60 solve) bit for
bit; the finest level's motion field is the solve's output; coarser levels'
motion fields follow computeMotionField (pdflow_cudalib.cu:1150-1167) at that
level, with the focal length of the finest solved width.
"""
import numpy as np
import pytest

from pdflow import BatchSolver, Solver, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("form", [5, 7, 8, 9, 10])
def test_level_record_equals_the_reference_levels(golden_qvga, form):
    g = golden_qvga
    s = Solver(60, 320, 240, iteration_form=form).initializeCUDA()
    s.keep_level_solutions(True)
    s.loadRGBDFrames(g["i1"], g["z1"], g["i2"], g["z2"])
    s.solveSceneFlowGPU()
    for level in range(3):
        rec = s.level_flow(level)
        for c in ("du", "dv", "dw"):
            ref = g[f"r60_{c}_l_L{level}"]
            assert np.array_equal(rec[c].view(np.uint32), ref.view(np.uint32)), (level, c)
    fin = s.level_flow(2)
    for c, out in zip(("dx", "dy", "dz"), (s.dxp, s.dyp, s.dzp)):
        assert np.array_equal(fin[c].view(np.uint32), out.view(np.uint32)), c
        assert np.array_equal(fin[c].view(np.uint32), g[f"r60_{c}"].view(np.uint32)), c
    s.freeGPUMemory()


def test_level_solutions_carry_the_level_images_and_motion_field(golden_qvga):
    g = golden_qvga
    s = Solver(60, 320, 240).initializeCUDA()
    s.keep_level_solutions(True)
    s.loadRGBDFrames(g["i1"], g["z1"], g["i2"], g["z2"])
    s.solveSceneFlowGPU()
    fovh = np.float64(np.float32(62.5 * np.pi / 180.0))   # the reference's default fovh
    cols = 80
    for level in range(3):
        sol = s.level_solutions(level)
        rec = s.level_flow(level)
        r, c = s.level_shape(level)
        assert sol["dx"].shape == (r * c,)
        # the record's motion field is what copyAllSolutions returns
        for k in ("dx", "dy", "dz"):
            assert np.array_equal(sol[k].view(np.uint32), rec[k].view(np.uint32)), (level, k)
        # computeMotionField at this level from the reference's own du_l, dv_l, dw_l
        z, xx, yy = (sol[k].astype(np.float64) for k in ("depth_old", "xx_old", "yy_old"))
        du, dv, dw = (g[f"r60_{k}_l_L{level}"].astype(np.float64) for k in ("du", "dv", "dw"))
        inv_f = 2.0 * np.tan(0.5 * fovh) / cols
        ok = z > 0
        zs = np.where(ok, z, 1.0)
        want = {"dx": np.where(ok, dw, 0.0), "dy": np.where(ok, z * du * inv_f + dw * xx / zs, 0.0),
                "dz": np.where(ok, z * dv * inv_f + dw * yy / zs, 0.0)}
        for k in ("dx", "dy", "dz"):
            np.testing.assert_allclose(sol[k], want[k], rtol=1e-5, atol=1e-7, err_msg=f"{level} {k}")
        # the images are the pyramid level that solved level uses (rows 60 of a
        # 320x240 frame: solved level i lives in pyramid image 4 - i)
        assert r == 240 >> (4 - level) and c == 320 >> (4 - level)
    s.freeGPUMemory()


def test_batch_records_every_pair_and_turning_it_off_keeps_the_bits():
    pairs = [scenes.make_pair(300 + k) for k in range(3)]
    b = BatchSolver(120, 320, 240, 3)
    b.push_raw(np.stack([p[0] for p in pairs]), np.stack([p[1] for p in pairs]))
    b.push_raw(np.stack([p[2] for p in pairs]), np.stack([p[3] for p in pairs]))
    b.solve(3)
    plain = b.read_flow(3)
    b.keep_level_solutions(True)
    b.solve(3)
    kept = b.read_flow(3)
    for x, y in zip(plain, kept):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    for k in range(3):
        fin = b.level_flow(3, pair=k)
        for c, name in enumerate(("dx", "dy", "dz")):
            assert np.array_equal(fin[name].view(np.uint32), kept[c][k].view(np.uint32)), (k, name)
    b.keep_level_solutions(False)
    b.solve(3)
    again = b.read_flow(3)
    for x, y in zip(plain, again):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    b.close()
