"""Mixed-resolution batches: pairs of rows 60/120/240/480 in one handle, one
launch per kernel per level size; every pair equals its single-pair solve."""
import numpy as np
import pytest

from pdflow import MixedBatch, Solver, scenes

pytestmark = pytest.mark.gpu


def single(rows, frames):
    i1, z1, i2, z2 = frames
    h, w = i1.shape
    s = Solver(rows, w, h).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    s.solveSceneFlowGPU()
    out = [x.copy() for x in (s.dxp, s.dyp, s.dzp)]
    s.freeGPUMemory()
    return out


@pytest.mark.parametrize("use_graph", [True, False])
def test_mixed_batch_pairs_equal_single_solves(built_lib, use_graph):
    rows = [60, 480, 240, 120, 480, 60, 240, 120, 30]
    pairs = [scenes.make_pair(600 + k, vga=(r == 480), n_objects=1 + k % 6) for k, r in enumerate(rows)]
    b = MixedBatch(12, use_graph=use_graph)
    b.push(rows, [p[0] for p in pairs], [p[1] for p in pairs])
    b.push(rows, [p[2] for p in pairs], [p[3] for p in pairs])
    for _ in range(2):                      # the replayed graph gives the same bits
        b.solve()
        for k, r in enumerate(rows):
            got = b.flow(k)
            ref = single(r, pairs[k])
            for x, y in zip(got, ref):
                assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (k, r)
    b.close()


def test_autotuned_mixed_batch_pairs_equal_single_solves(built_lib):
    """The autotuner picks a tile form and iterations per launch per
    coarse-to-fine step over the pairs active there; the tuned plan still gives
    every pair its single-pair solve, bit for bit."""
    rows = [480, 60, 240, 120, 480, 240, 30]
    pairs = [scenes.make_pair(700 + k, vga=(r == 480), n_objects=1 + k % 5) for k, r in enumerate(rows)]
    b = MixedBatch(8)
    b.push(rows, [p[0] for p in pairs], [p[1] for p in pairs])
    b.push(rows, [p[2] for p in pairs], [p[3] for p in pairs])
    rep = b.autotune()
    assert [r["step"] for r in rep] == ["15x20", "30x40", "60x80", "120x160", "240x320", "480x640"]
    for r in rep:
        assert (r["form"], r["iters_per_launch"]) in [(f, k) for f in (3, 4, 5, 6, 7, 8, 10) for k in (2, 3, 4)] + [
            (9, 4), (9, 6), (9, 8)]
        assert r["ms_per_iter"][0] is None                      # two kernels per iteration: not a mixed form
        if r["step"] == "15x20":
            assert r["form"] <= 6                                # odd rows: no register tiles
        if r["step"] == "30x40":
            assert r["form"] not in (7, 10)                      # rows % 4 != 0: no tensor-copy tiles
    for _ in range(2):                                           # graph capture, then replay
        b.solve()
        for k, r in enumerate(rows):
            got = b.flow(k)
            ref = single(r, pairs[k])
            for x, y in zip(got, ref):
                assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (k, r)
    b.close()


def test_mixed_batch_rejects_bad_rows(built_lib):
    from pdflow import ERR_ARG, PDFlowError
    b = MixedBatch(2)
    i, z = scenes.make_pair(1)[:2]
    with pytest.raises(PDFlowError) as e:
        b.push([100], [i], [z])
    assert e.value.code == ERR_ARG
    b.close()


def test_regular_calls_are_refused_on_a_mixed_handle(built_lib):
    """A mixed-resolution handle answers PDFLOW_ERR_STATE to the single-shape
    push / solve / read calls (its pairs have per-pair shapes)."""
    from pdflow import _lib
    lib = _lib.load()
    import ctypes
    h = ctypes.c_void_p()
    assert lib.pdflow_create_mixed(4, ctypes.byref(h)) == _lib.OK
    buf = np.zeros(640 * 480 * 4, np.float32)
    assert lib.pdflow_solve_batch(h, 1) == _lib.ERR_STATE
    assert lib.pdflow_push_frames(h, 1, buf.ctypes.data_as(ctypes.c_void_p), buf.ctypes.data_as(ctypes.c_void_p)) \
        == _lib.ERR_STATE
    assert lib.pdflow_read_flow_batch(h, 1, *[buf.ctypes.data_as(ctypes.c_void_p)] * 3) == _lib.ERR_STATE
    assert "mixed" in _lib.last_error()
    assert lib.pdflow_destroy(h) == _lib.OK
