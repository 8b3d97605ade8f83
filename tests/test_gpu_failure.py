"""Failure detection without a GPU fault: a bounded device-side wait on a
progress counter that nothing sets runs out, the kernel records the timeout
in the handle's status word and returns, the host reports
PDFLOW_ERR_TIMEOUT, and the same handle then solves correctly."""
import numpy as np
import pytest

from pdflow import Solver, _lib, scenes

pytestmark = pytest.mark.gpu


def test_wait_timeout_is_reported_and_the_handle_stays_usable(built_lib):
    lib = _lib.load()
    i1, z1, i2, z2 = scenes.make_pair(3)
    ref = Solver(240, 320, 240).initializeCUDA()
    ref.loadRGBDFrames(i1, z1, i2, z2)
    ref.solveSceneFlowGPU()

    s = Solver(240, 320, 240).initializeCUDA()
    assert lib.pdflow_debug_wait_timeout(s._h, 0) == _lib.ERR_ARG
    for _ in range(2):   # twice: the status word is reset after each report
        assert lib.pdflow_debug_wait_timeout(s._h, 1000) == _lib.ERR_TIMEOUT
        assert "bounded device-side wait" in _lib.last_error()
    s.loadRGBDFrames(i1, z1, i2, z2)
    s.solveSceneFlowGPU()
    for a, b in zip((s.dxp, s.dyp, s.dzp), (ref.dxp, ref.dyp, ref.dzp)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.abs(s.dxp).max() > 0
    s.freeGPUMemory()
    ref.freeGPUMemory()
