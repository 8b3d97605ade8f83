"""The bench's headline workload at full size: a 64-pair VGA batch (rows 480,
1-8 objects per scene), autotuned, equals 64 single-pair solves bit for bit."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_64_vga_pairs_autotuned_equal_single_solves(built_lib):
    torch = pytest.importorskip("torch")
    from pdflow import BatchSolver, Solver, _lib, datagen
    n = 64
    seeds = list(range(4_100_000, 4_100_000 + n))
    i1, z1, i2, z2 = datagen.render_pairs(torch, seeds, True, n_objects=lambda s: 1 + s % 8)
    torch.cuda.synchronize()
    b = BatchSolver(480, 640, 480, n)
    b.push_raw_device(n, i1.data_ptr(), z1.data_ptr())
    b.push_raw_device(n, i2.data_ptr(), z2.data_ptr())
    tune = b.autotune(n)
    assert [t["form"] for t in tune][-1] in range(3, 11)
    b.solve(n)
    got = b.read_flow(n)
    b.close()
    lib = _lib.load()
    s = Solver(480, 640, 480).initializeCUDA()
    p = ctypes.c_void_p
    for k in range(n):
        _lib.check(lib.pdflow_push_frame_u16_device(s.handle, p(i1[k].data_ptr()), p(z1[k].data_ptr())), "push")
        _lib.check(lib.pdflow_push_frame_u16_device(s.handle, p(i2[k].data_ptr()), p(z2[k].data_ptr())), "push")
        s.solveSceneFlowGPU()
        for c, one in enumerate((s.dxp, s.dyp, s.dzp)):
            assert np.array_equal(got[c][k].view(np.uint32), one.view(np.uint32)), (k, c)
    s.freeGPUMemory()
