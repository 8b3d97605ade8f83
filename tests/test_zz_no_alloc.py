"""The allocation-free entry point pdflow_solve_pair_noalloc.

Callers that may not allocate device memory once they are running (a
real-time camera loop with a fixed memory budget, a plugin whose host framework
owns every allocation) solve a pair with scratch memory compiled into the
library instead of a per-handle arena.  Its result must equal the regular entry
point's on the same frames, including on a second call that reuses the scratch
left behind by the first.

This file is collected last (test_zz_*), so a stop-at-first-failure run has
run every other test before it; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from pdflow import Solver, scenes

pytestmark = pytest.mark.gpu

FLOW_MEAN_TOL = 1e-4   # metres, as the parity tests
FLOW_MAX_TOL = 1e-3


def regular(rows, frames):
    i1, z1, i2, z2 = frames
    h, w = i1.shape
    s = Solver(rows, w, h).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    s.solveSceneFlowGPU()
    out = [x.copy() for x in (s.dxp, s.dyp, s.dzp)]
    s.freeGPUMemory()
    return out


def device_buffers(torch, rows, frames):
    """The caller's own device buffers: both frames and the three flow planes."""
    i1, z1, i2, z2 = frames
    cols = rows * 320 // 240
    dev = [torch.from_numpy(np.ascontiguousarray(a.view(np.int16) if a.dtype == np.uint16 else a)).cuda()
           for a in (i1, z1, i2, z2)]
    out = [torch.full((rows * cols,), float("nan"), dtype=torch.float32, device="cuda") for _ in range(3)]
    return dev, out


def call_noalloc(lib, torch, rows, frames, dev, out):
    h, w = frames[0].shape
    stream = torch.cuda.current_stream()
    rc = lib.pdflow_solve_pair_noalloc(rows, w, h, None, *[ctypes.c_void_p(t.data_ptr()) for t in dev + out],
                                       ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.pdflow_last_error()
    torch.cuda.synchronize()


def noalloc(lib, torch, rows, frames):
    dev, out = device_buffers(torch, rows, frames)
    call_noalloc(lib, torch, rows, frames, dev, out)
    return [t.cpu().numpy() for t in out]


def check(a, b):
    for x, y in zip(a, b):
        d = np.abs(x.astype(np.float64) - y)
        assert d.mean() <= FLOW_MEAN_TOL and d.max() <= FLOW_MAX_TOL
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))   # same kernels: same bits


@pytest.mark.parametrize("rows", [120, 60])
def test_noalloc_matches_regular_entry_point_on_two_calls_in_a_row(built_lib, rows):
    torch = pytest.importorskip("torch")
    first = scenes.make_pair(31, vga=False, n_objects=3)
    second = scenes.make_pair(32, vga=False, n_objects=5)
    got1 = noalloc(built_lib, torch, rows, first)
    got2 = noalloc(built_lib, torch, rows, second)   # scratch still holds the first call's state
    check(got1, regular(rows, first))
    check(got2, regular(rows, second))


def test_noalloc_rejects_configurations_beyond_its_scratch(built_lib):
    torch = pytest.importorskip("torch")
    from pdflow import ERR_ARG
    buf = torch.zeros(640 * 480, dtype=torch.int16, device="cuda")
    out = torch.zeros(480 * 640, dtype=torch.float32, device="cuda")
    p = ctypes.c_void_p
    rc = built_lib.pdflow_solve_pair_noalloc(240, 320, 240, None, p(buf.data_ptr()), p(buf.data_ptr()),
                                             p(buf.data_ptr()), p(buf.data_ptr()), p(out.data_ptr()),
                                             p(out.data_ptr()), p(out.data_ptr()), None)
    assert rc == ERR_ARG
    assert b"scratch" in built_lib.pdflow_last_error()


def test_noalloc_calls_after_the_first_allocate_no_device_memory(built_lib):
    """The property the entry point exists for: once the first call on the
    device has loaded the scratch array, further calls change neither the
    device's free memory (cudaMemGetInfo) nor torch's allocator statistics."""
    torch = pytest.importorskip("torch")
    frames = [scenes.make_pair(33 + k, vga=False, n_objects=3) for k in range(2)]
    bufs = [device_buffers(torch, 120, f) for f in frames]
    call_noalloc(built_lib, torch, 120, frames[0], *bufs[0])   # first call: one-time set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    stats0 = torch.cuda.memory_stats()
    for f, b in zip(frames, bufs):
        call_noalloc(built_lib, torch, 120, f, *b)
    free1, _ = torch.cuda.mem_get_info()
    stats1 = torch.cuda.memory_stats()
    assert free1 == free0
    for key in ("allocation.all.allocated", "reserved_bytes.all.current", "allocated_bytes.all.current"):
        assert stats1.get(key, 0) == stats0.get(key, 0), key
