"""Parity of the sm_103a solver (called through the C ABI) with the reference's
own CUDA path (golden vectors) and with the CPU oracle.

The solver reproduces the reference's CUDA path bit for bit (every stage and
the final flow).  The stated floating-point tolerance (mean |d| <= 1e-4 m,
max |d| <= 1e-3 m) is checked as well, so that a failure of exactness is
reported against the tolerance the flow must always meet.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from pdflow import Solver, scenes

pytestmark = pytest.mark.gpu

FLOW_MEAN_TOL = 1e-4
FLOW_MAX_TOL = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def solve(g, rows, w, h, raw=True, graph=True, debug=False, form=1):
    s = Solver(rows, w, h, use_graph=graph, iteration_form=form).initializeCUDA()
    try:
        if raw:
            s.loadRGBDFrames(g["i1"], g["z1"], g["i2"], g["z2"])
        else:
            for a, b in (("i1", "z1"), ("i2", "z2")):
                I, Z = scenes.decode(g[a], g[b])
                s.createImagePyramidGPU(I, Z)
        if debug:
            st = s.debug_solve()
            return [x.copy() for x in (s.dxp, s.dyp, s.dzp)], st, s
        s.solveSceneFlowGPU()
        return [x.copy() for x in (s.dxp, s.dyp, s.dzp)]
    finally:
        if not debug:
            s.freeGPUMemory()


CASES = [("qvga_s0.npz", 240, 320, 240), ("qvga_s0.npz", 60, 320, 240),
         ("vga_s2.npz", 480, 640, 480), ("vga_s2.npz", 240, 640, 480)]


@pytest.mark.parametrize("form", [1, 7, 8, 9, 10])
@pytest.mark.parametrize("fixture,rows,w,h", CASES)
def test_flow_matches_reference_cuda_path(fixture, rows, w, h, form):
    """The final flow equals the reference's own CUDA build bit for bit, with
    the level iterations as one persistent launch (form 1) or as register-
    resident quad tiles (form 7)."""
    from conftest import load_golden
    g = load_golden(fixture)
    out = solve(g, rows, w, h, form=form)
    for c, o in zip(("dx", "dy", "dz"), out):
        ref = g[f"r{rows}_{c}"]
        d = np.abs(o.astype(np.float64) - ref)
        exact = float(np.mean(o.view(np.uint32) == ref.view(np.uint32)))
        print(f"{fixture} rows={rows} {c}: mean {d.mean():.3e} max {d.max():.3e} bit-exact {exact:.4f}")
        assert d.mean() <= FLOW_MEAN_TOL, (c, d.mean())
        assert d.max() <= FLOW_MAX_TOL, (c, d.max())
        assert exact == 1.0, (c, exact)


@pytest.mark.parametrize("fixture,rows,w,h", CASES[:3])
def test_flow_tracks_fp64_oracle(fixture, rows, w, h):
    from conftest import load_golden
    g = load_golden(fixture)
    out = solve(g, rows, w, h)
    I1, Z1 = scenes.decode(g["i1"], g["z1"])
    I2, Z2 = scenes.decode(g["i2"], g["z2"])
    ref = oracle.solve(rows, w, h, I1, Z1, I2, Z2, precision="f64")
    for o, r in zip(out, ref):
        d = np.abs(o.astype(np.float64) - r)
        assert d.mean() <= 1e-5
        assert float((d > 1e-3).mean()) <= 1e-4


def test_pyramid_is_bit_exact_with_reference(golden_qvga):
    """Both frames' pyramid levels 2..4 (80x60 .. 20x15) equal the reference's bit for bit."""
    g = golden_qvga
    s = Solver(60, 320, 240).initializeCUDA()
    s.loadRGBDFrames(g["i1"], g["z1"], g["i2"], g["z2"])
    for lv in (2, 3, 4):
        for frame, pre in ((0, "old_push_"), (1, "push_")):
            imgs = s.level_images(lv, frame)
            for fld in ("colour", "depth", "xx", "yy"):
                ref = g[f"r60_{pre}{fld}_L{lv}"]
                assert np.array_equal(imgs[fld].view(np.uint32), ref.view(np.uint32)), (lv, frame, fld)
    s.freeGPUMemory()


@pytest.mark.parametrize("vga", [False, True])
def test_device_decode_is_bit_exact(vga):
    i1, z1, i2, z2 = scenes.make_pair(11, vga=vga)
    h, w = i1.shape
    s = Solver(240, w, h).initializeCUDA()
    s.loadRGBDFrames(i1, z1, i2, z2)
    for frame, (ii, zz) in ((0, (i1, z1)), (1, (i2, z2))):
        I, Z = oracle.decode_frame(ii, zz)
        imgs = s.level_images(0, frame)
        assert np.array_equal(imgs["colour"].view(np.uint32), I.view(np.uint32))
        assert np.array_equal(imgs["depth"].view(np.uint32), Z.view(np.uint32))
    s.freeGPUMemory()


SETUP = ("dct", "dcu", "dcv", "ddt", "ddu", "ddv", "mu", "ri", "rj", "ri_2", "rj_2", "sigma_pd", "sigma_puvx",
         "sigma_puvy", "sigma_pwx", "sigma_pwy", "tau_u", "tau_v", "tau_w")


@pytest.fixture(scope="module")
def debug_r60(golden_qvga):
    out, st, s = solve(golden_qvga, 60, 320, 240, debug=True)
    s.freeGPUMemory()
    return out, st


def test_debug_solve_equals_solve(golden_qvga, debug_r60):
    out = solve(golden_qvga, 60, 320, 240)
    for a, b in zip(out, debug_r60[0]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("field", SETUP)
def test_coarsest_level_setup_matches_reference(golden_qvga, debug_r60, field):
    """Same pyramid in, same set-up out: the coarsest level's set-up fields
    agree with the reference's to within FP32 rounding (bit-exact when nvcc
    forms the same fused multiply-adds)."""
    ours = debug_r60[1][(field, 0)]
    ref = golden_qvga[f"r60_{field}_L0"]
    exact = float(np.mean(ours.view(np.uint32) == ref.view(np.uint32)))
    print(f"{field}: bit-exact fraction {exact:.4f}")
    assert np.allclose(ours, ref, rtol=1e-5, atol=1e-7), field
    assert exact == 1.0, field


@pytest.mark.parametrize("field", ("du_l", "dv_l", "dw_l", "sat_du", "pd", "puu"))
@pytest.mark.parametrize("level", (0, 1, 2))
def test_level_state_matches_reference(golden_qvga, debug_r60, field, level):
    ours = debug_r60[1][(field, level)]
    ref = golden_qvga[f"r60_{field}_L{level}"]
    d = np.abs(ours.astype(np.float64) - ref)
    print(f"{field} L{level}: max {d.max():.3e} bit-exact {np.mean(ours.view(np.uint32) == ref.view(np.uint32)):.4f}")
    assert d.mean() <= 1e-5 and d.max() <= 1e-3
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32)), (field, level)


def test_median_selection_is_bit_exact_with_oracle(golden_qvga, built_lib):
    """Weighted-median selection (filterSolution) on identical inputs picks the
    same bracketing sample as the oracle for every pixel and component."""
    torch = pytest.importorskip("torch")
    g = golden_qvga
    R, C = 60, 80
    depth = g["r60_old_push_depth_L2"].astype(np.float32)
    ddt = g["r60_ddt_L2"].astype(np.float32)
    du, dv, dw = (g[f"r60_sat_{c}_L2"].astype(np.float32) for c in ("du", "dv", "dw"))
    # force exact ties in dw (common in practice: dw = 0 beside holes)
    dw = dw.copy()
    dw[::7] = 0.0
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    t_in = [dev(a) for a in (depth, ddt, du, dv, dw)]
    t_out = [torch.zeros(R * C, dtype=torch.float32, device="cuda") for _ in range(3)]
    t_sel = torch.zeros(3 * R * C, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    rc = built_lib.pdflow_stage_median(R, C, *[ctypes.c_void_p(t.data_ptr()) for t in t_in + t_out],
                                       ctypes.c_void_p(t_sel.data_ptr()), ctypes.c_void_p(st))
    assert rc == 0
    torch.cuda.synchronize()
    o = [np.zeros(R * C, np.float32) for _ in range(3)]
    sel = np.zeros(3 * R * C, np.int32)
    oracle.stage_call("median", "f32", R, C, depth, ddt, du, dv, dw, o[0], o[1], o[2], sel)
    gsel = t_sel.cpu().numpy()
    assert np.array_equal(gsel, sel)
    for a, b in zip(t_out, o):
        assert np.allclose(a.cpu().numpy(), b, rtol=1e-6, atol=1e-7)


def test_solve_is_deterministic(golden_qvga):
    a = solve(golden_qvga, 240, 320, 240)
    b = solve(golden_qvga, 240, 320, 240)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_graph_and_stream_forms_agree(golden_qvga):
    a = solve(golden_qvga, 120, 320, 240, graph=True)
    b = solve(golden_qvga, 120, 320, 240, graph=False)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.parametrize("fixture,rows,w,h", [CASES[0], CASES[2]])
def test_iteration_forms_agree(fixture, rows, w, h):
    """Temporally blocked tiles (scalar, paired, register-resident quads),
    one launch per level's iterations (slab-persistent kernel) and two kernels
    per iteration give the same bits."""
    from conftest import load_golden
    g = load_golden(fixture)
    a = solve(g, rows, w, h, form=2)
    for form in (1, 0, 5, 7, 8, 9, 10):
        b = solve(g, rows, w, h, form=form)
        for x, y in zip(a, b):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), form


def test_float_and_raw_pushes_agree(golden_qvga):
    a = solve(golden_qvga, 120, 320, 240, raw=True)
    b = solve(golden_qvga, 120, 320, 240, raw=False)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_repeated_pairs_on_one_handle(golden_qvga):
    """A handle solves pair after pair; each push shifts new -> old like the
    reference's pointer swap (pdflow_cudalib.cu:203-221)."""
    g = golden_qvga
    s = Solver(60, 320, 240).initializeCUDA()
    s.push_raw(g["i2"], g["z2"])   # stale frame, pushed out below
    s.push_raw(g["i1"], g["z1"])
    s.push_raw(g["i2"], g["z2"])
    s.solveSceneFlowGPU()
    first = [x.copy() for x in (s.dxp, s.dyp, s.dzp)]
    s.push_raw(g["i1"], g["z1"])
    s.push_raw(g["i2"], g["z2"])
    s.solveSceneFlowGPU()
    for x, y in zip(first, (s.dxp, s.dyp, s.dzp)):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    ref = g["r60_dx"]
    assert np.abs(first[0] - ref).max() <= FLOW_MAX_TOL
    s.freeGPUMemory()


def test_solve_before_two_frames_is_a_state_error(built_lib):
    from pdflow import ERR_STATE, PDFlowError
    s = Solver(60, 320, 240).initializeCUDA()
    with pytest.raises(PDFlowError) as e:
        s.solveSceneFlowGPU()
    assert e.value.code == ERR_STATE
    s.freeGPUMemory()


def test_zero_iteration_schedule_still_saturates_and_filters(golden_qvga):
    from pdflow import default_params
    p = default_params(60)
    for i in range(6):
        p.num_max_iter[i] = 0
    g = golden_qvga
    s = Solver(60, 320, 240, params=p).initializeCUDA()
    s.loadRGBDFrames(g["i1"], g["z1"], g["i2"], g["z2"])
    s.solveSceneFlowGPU()
    I1, Z1 = scenes.decode(g["i1"], g["z1"])
    I2, Z2 = scenes.decode(g["i2"], g["z2"])
    ref = oracle.solve(60, 320, 240, I1, Z1, I2, Z2, precision="f32", iters=[0] * 6)
    for o, r in zip((s.dxp, s.dyp, s.dzp), ref):
        assert np.allclose(o, r, atol=1e-6)
    s.freeGPUMemory()


def test_all_solutions_readback_matches_the_parts(golden_qvga):
    """pdflow_read_all_solutions (copyAllSolutions) returns the flow and both
    frames' images of the finest solved level."""
    g = golden_qvga
    s = Solver(60, 320, 240).initializeCUDA()
    s.loadRGBDFrames(g["i1"], g["z1"], g["i2"], g["z2"])
    s.solveSceneFlowGPU()
    out = s.all_solutions()
    for a, b in zip((out["dx"], out["dy"], out["dz"]), (s.dxp, s.dyp, s.dzp)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    new, old = s.level_images(2, 1), s.level_images(2, 0)      # 80x60 = rows 60 x cols 80
    for k in ("depth", "colour", "xx", "yy"):
        assert np.array_equal(out[k], new[k]) and np.array_equal(out[k + "_old"], old[k])
    s.freeGPUMemory()


def test_reciprocal_division_equals_ieee_division():
    """The register tiles' shrinkage divides by the pixel's fixed denominator
    through its correctly rounded reciprocal and two FMA corrections
    (Markstein); on 2^28 random pairs of the range it is used in (and signed
    zeros, and denominators at the 1e-10 floor) it gives the bits of the IEEE
    division the reference performs (pdflow_cudalib.cu:921-922)."""
    from pdflow import _lib
    lib = _lib.load()
    bad = ctypes.c_ulonglong(1)
    assert lib.pdflow_check_div_rcp(1 << 28, 20261204, ctypes.byref(bad)) == 0
    assert bad.value == 0
