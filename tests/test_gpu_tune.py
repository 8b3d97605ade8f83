"""The launch-form autotuner: every candidate gives the same bits, and the
tuned handle still solves bit-exactly."""
import numpy as np
import pytest

from pdflow import BatchSolver, scenes

pytestmark = pytest.mark.gpu


def test_autotuned_forms_give_the_same_bits(built_lib):
    import ctypes
    from pdflow import _lib
    pairs = [scenes.make_pair(900 + k) for k in range(3)]
    b = BatchSolver(240, 320, 240, 3)
    b.push_raw(np.stack([p[0] for p in pairs]), np.stack([p[1] for p in pairs]))
    b.push_raw(np.stack([p[2] for p in pairs]), np.stack([p[3] for p in pairs]))
    b.solve(3)
    ref = b.read_flow(3)

    lib = _lib.load()
    rep = b.autotune(3)
    assert len(rep) == 5
    for lvl in rep:
        assert lvl["form"] in range(11)
        assert lvl["ms_per_iter"][0] is not None
    b.solve(3)
    got = b.read_flow(3)
    for x, y in zip(got, ref):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    # each tile width of iterations per launch, forced on every level
    for form, kk in ((2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (3, 3), (3, 4), (4, 1), (4, 3), (4, 4), (7, 1), (7, 2),
                     (7, 3), (7, 4), (8, 1), (8, 2), (8, 3), (8, 4), (9, 1), (9, 3), (9, 5), (9, 8),
                     (10, 1), (10, 2), (10, 3), (10, 4)):
        for lvl in range(5):
            assert lib.pdflow_set_level_form(b.handle, lvl, form, kk) == 0
        b.solve(3)
        got = b.read_flow(3)
        for x, y in zip(got, ref):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    b.close()


DEFAULT_COPY_MODE = {3: 5, 4: 5, 5: 5, 6: 5}   # the library's defaults (pdflow_tiles2.cu)


@pytest.mark.parametrize("form", [3, 4, 5, 6])
def test_tile_copy_modes_give_the_same_bits(built_lib, form):
    import ctypes
    from pdflow import _lib
    lib = _lib.load()
    n = 4
    pairs = [scenes.make_pair(950 + k) for k in range(n)]
    out = []
    for mode in (0, 1, 2, 3, 5, 7):   # plain, bulk and tensor-copy loads, plain and bulk stores
        assert lib.pdflow_set_tile_copy_mode(form - 3, mode) == 0
        b = BatchSolver(240, 320, 240, n, iteration_form=form)
        b.push_raw(np.stack([p[0] for p in pairs]), np.stack([p[1] for p in pairs]))
        b.push_raw(np.stack([p[2] for p in pairs]), np.stack([p[3] for p in pairs]))
        b.solve(n)
        out.append(b.read_flow(n))
        b.close()
    lib.pdflow_set_tile_copy_mode(form - 3, DEFAULT_COPY_MODE[form])
    for o in out[1:]:
        for x, y in zip(o, out[0]):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
