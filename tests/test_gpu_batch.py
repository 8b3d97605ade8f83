"""Batches: every pair of a batch equals its single-pair solve, bit for bit."""
import numpy as np
import pytest

from pdflow import BatchSolver, Solver, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def single(rows, frames, form=1):
    i1, z1, i2, z2 = frames
    h, w = i1.shape
    s = Solver(rows, w, h, iteration_form=form).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    s.solveSceneFlowGPU()
    out = [x.copy() for x in (s.dxp, s.dyp, s.dzp)]
    s.freeGPUMemory()
    return out


def batch_solve(rows, pairs, capacity=None, form=1):
    h, w = pairs[0][0].shape
    n = len(pairs)
    b = BatchSolver(rows, w, h, capacity or n, iteration_form=form)
    b.push_raw(np.stack([p[0] for p in pairs]), np.stack([p[1] for p in pairs]))
    b.push_raw(np.stack([p[2] for p in pairs]), np.stack([p[3] for p in pairs]))
    b.solve(n)
    out = b.read_flow(n)
    b.close()
    return out


@pytest.mark.parametrize("vga,rows,n", [(False, 240, 4), (False, 60, 5), (True, 480, 3), (True, 240, 2)])
def test_batch_pairs_equal_single_solves(vga, rows, n):
    pairs = [scenes.make_pair(100 + k, vga=vga, n_objects=1 + (k % 8)) for k in range(n)]
    got = batch_solve(rows, pairs)
    for k, fr in enumerate(pairs):
        ref = single(rows, fr)
        for c in range(3):
            assert np.array_equal(got[c][k].view(np.uint32), ref[c].view(np.uint32)), (k, c)


def test_partial_batch_and_golden(golden_qvga):
    """Solving n < capacity pairs; pair 0 fed the golden frames reproduces the
    reference's CUDA output."""
    g = golden_qvga
    pairs = [(g["i1"], g["z1"], g["i2"], g["z2"]), scenes.make_pair(7)]
    got = batch_solve(240, pairs, capacity=6)
    for c, name in enumerate(("dx", "dy", "dz")):
        assert np.array_equal(got[c][0].view(np.uint32), g[f"r240_{name}"].view(np.uint32))


@pytest.mark.parametrize("vga,rows", [(False, 120), (False, 240), (True, 480)])
def test_batch_iteration_forms_agree(vga, rows):
    pairs = [scenes.make_pair(200 + k, vga=vga) for k in range(3)]
    a = batch_solve(rows, pairs, form=2)
    for form in (3, 4, 5, 6, 7, 8, 9, 10, 1, 0):
        b = batch_solve(rows, pairs, form=form)
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), form


def test_batch_rejects_bad_counts():
    from pdflow import ERR_ARG, PDFlowError
    b = BatchSolver(60, 320, 240, 2)
    with pytest.raises(PDFlowError) as e:
        b.solve(3)
    assert e.value.code == ERR_ARG
    b.close()


def test_trace_solve_times_every_phase_and_keeps_the_flow(built_lib):
    """pdflow_trace_solve: per-level set-up / iterations / median times of an
    eager solve, whose flow is the plain solve's bit for bit."""
    pairs = [scenes.make_pair(400 + k) for k in range(2)]
    b = BatchSolver(240, 320, 240, 2)
    b.push_raw(np.stack([p[0] for p in pairs]), np.stack([p[1] for p in pairs]))
    b.push_raw(np.stack([p[2] for p in pairs]), np.stack([p[3] for p in pairs]))
    b.solve(2)
    ref = b.read_flow(2)
    tr = b.trace(2)
    got = b.read_flow(2)
    b.close()
    assert len(tr) == 5
    for t in tr:
        assert t["setup_ms"] > 0 and t["iterations_ms"] > 0 and t["median_ms"] > 0
    assert tr[-1]["iterations_ms"] > tr[0]["iterations_ms"]      # 100 iterations at 240x320 vs 40 at 15x20
    for x, y in zip(got, ref):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_repeated_solves_are_bit_identical(built_lib):
    """Determinism: the same frames solved twice (graph replay and an eager
    stream of kernels) give the same bits."""
    pairs = [scenes.make_pair(410 + k, vga=True) for k in range(2)]
    out = []
    for graph in (True, True, False):
        b = BatchSolver(480, 640, 480, 2, use_graph=graph)
        b.push_raw(np.stack([p[0] for p in pairs]), np.stack([p[1] for p in pairs]))
        b.push_raw(np.stack([p[2] for p in pairs]), np.stack([p[3] for p in pairs]))
        b.solve(2)
        b.solve(2)
        out.append(b.read_flow(2))
        b.close()
    for o in out[1:]:
        for x, y in zip(o, out[0]):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_copy_flow_device_matches_read_flow(built_lib):
    """pdflow_copy_flow_device: all pairs' flows into contiguous device buffers."""
    torch = pytest.importorskip("torch")
    import ctypes
    from pdflow import _lib
    pairs = [scenes.make_pair(420 + k) for k in range(3)]
    b = BatchSolver(120, 320, 240, 4)
    b.push_raw(np.stack([p[0] for p in pairs]), np.stack([p[1] for p in pairs]))
    b.push_raw(np.stack([p[2] for p in pairs]), np.stack([p[3] for p in pairs]))
    b.solve(3)
    ref = b.read_flow(3)
    out = torch.zeros((3, 3, 120 * 160), dtype=torch.float32, device="cuda")
    assert _lib.load().pdflow_copy_flow_device(b.handle, 3, *[ctypes.c_void_p(out[c].data_ptr()) for c in range(3)]) == 0
    b.synchronize()
    got = out.cpu().numpy()
    b.close()
    for c in range(3):
        assert np.array_equal(got[c].view(np.uint32), ref[c].view(np.uint32))
