"""Slot-addressed batches, the energy functional and the seeded (warm-started)
level schedule on the GPU, against single solves and the CPU oracle."""
import numpy as np
import pytest

from oracle import oracle
from pdflow import ERR_ARG, ERR_STATE, BatchSolver, PDFlowError, Solver, scenes

pytestmark = pytest.mark.gpu

FLOW_MEAN_TOL = 1e-4   # metres
FLOW_MAX_TOL = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def single(rows, i1, z1, i2, z2):
    h, w = i1.shape
    s = Solver(rows, w, h).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    s.solveSceneFlowGPU()
    out = [x.copy() for x in (s.dxp, s.dyp, s.dzp)]
    s.freeGPUMemory()
    return out


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def test_slots_keep_each_streams_previous_frame():
    """Slot 2 sees frames A0, A1, A2 and slot 0 sees B0, B1, pushed in separate
    calls; each solve equals the single solve of that stream's last two frames."""
    from pdflow.scenes import make_scene, render
    sa, sb = make_scene(41, n_objects=3), make_scene(42, n_objects=5)
    A = [render(sa, k) for k in range(3)]
    B = [render(sb, k) for k in range(2)]
    b = BatchSolver(120, 320, 240, 4)
    b.push_slots([2], A[0][0][None], A[0][1][None])
    b.push_slots([2, 0], np.stack([A[1][0], B[0][0]]), np.stack([A[1][1], B[0][1]]))
    b.push_slots([0], B[1][0][None], B[1][1][None])
    b.solve_slots([2, 0])
    got = b.read_flow_slots([2, 0])
    ref_a = single(120, *A[0], *A[1])
    ref_b = single(120, *B[0], *B[1])
    for c in range(3):
        assert bits_equal(got[c][0], ref_a[c]) and bits_equal(got[c][1], ref_b[c])
    b.push_slots([2], A[2][0][None], A[2][1][None])
    b.solve_slots([2])
    got = b.read_flow_slots([2])
    ref = single(120, *A[1], *A[2])
    for c in range(3):
        assert bits_equal(got[c][0], ref[c])
    b.close()


def test_slot_calls_reject_bad_use():
    b = BatchSolver(60, 320, 240, 3)
    i1, z1, i2, z2 = scenes.make_pair(5)
    with pytest.raises(PDFlowError) as e:
        b.push_slots([1, 1], np.stack([i1, i2]), np.stack([z1, z2]))
    assert e.value.code == ERR_ARG
    b.push_slots([1], i1[None], z1[None])
    with pytest.raises(PDFlowError) as e:
        b.solve_slots([1])                      # one frame only
    assert e.value.code == ERR_STATE
    with pytest.raises(PDFlowError) as e:
        b.push_raw(i1[None], z1[None])          # whole-batch push on a slot handle
    assert e.value.code == ERR_STATE
    with pytest.raises(PDFlowError) as e:
        b.solve_slots([3])
    assert e.value.code == ERR_ARG
    b.close()


@pytest.mark.parametrize("rows", [240, 120])
def test_energy_matches_the_oracle_functional(rows):
    i1, z1, i2, z2 = scenes.make_pair(77, n_objects=3)
    s = Solver(rows, 320, 240).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    s.solveSceneFlowGPU()
    e_gpu = float(s.energy(1)[0])
    du, dv, dw = (a[0] for a in s.image_flow(1))
    cfg = s.config()
    li = 0 + int(np.log2(320 // s.cols))           # image level of the finest solved level
    old = s.level_images(li, 0)
    new = s.level_images(li, 1)
    key = ("colour", "depth", "xx", "yy")
    e_ref = oracle.energy(rows, s.cols, [old[k] for k in key], [new[k] for k in key], du, dv, dw)
    s.freeGPUMemory()
    assert cfg["rows"] == rows
    assert abs(e_gpu - e_ref) <= 2e-5 * e_ref, (e_gpu, e_ref)


@pytest.mark.parametrize("scale", [1.0, 0.5])
def test_seeded_levels_match_the_oracle(scale):
    torch = pytest.importorskip("torch")
    i1, z1, i2, z2 = scenes.make_pair(19, n_objects=4)
    I1, Z1 = scenes.decode(i1, z1)
    I2, Z2 = scenes.decode(i2, z2)
    _, _, _, st = oracle.solve(120, 320, 240, I1, Z1, I2, Z2, precision="f64", dump=True)
    seed = np.concatenate([st[(k, 2)] for k in ("du_l", "dv_l", "dw_l")]).astype(np.float32)
    rx, ry, rz = oracle.solve_seeded(120, 320, 240, I1, Z1, I2, Z2, 2, seed, scale)
    s = Solver(120, 320, 240).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    d_seed = torch.from_numpy(seed).cuda()
    s.solve_levels(1, 2, 99, d_seed.data_ptr(), scale)
    gx, gy, gz = s.read_flow()
    s.freeGPUMemory()
    for g, r in ((gx, rx), (gy, ry), (gz, rz)):
        d = np.abs(g.astype(np.float64) - r)
        assert d.mean() <= FLOW_MEAN_TOL and d.max() <= FLOW_MAX_TOL, (d.mean(), d.max())


def test_level_energy_of_plain_levels_is_reported():
    i1, z1, i2, z2 = scenes.make_pair(23)
    s = Solver(240, 320, 240).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    e = s.solve_levels(1, 0, 2, None, 1.0, 2)
    assert e is not None and np.isfinite(e[0]) and e[0] > 0
    with pytest.raises(PDFlowError) as err:
        s.solve_levels(1, 2, 4, None, 1.0)       # a level > 0 needs a seed
    assert err.value.code == ERR_ARG
    s.freeGPUMemory()
