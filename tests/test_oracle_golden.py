"""Pins the CPU oracle against the reference's own CUDA path.

The golden vectors in tests/golden/ were produced by the reference's unmodified
device code (pdflow_cudalib.cu built for sm_103a) driven through the host
sequence of PD_flow_opencv (tests/golden/make_golden.py).  The oracle is a
plain-C restatement without fused multiply-adds, so it matches the reference to
FP32 rounding in every set-up stage and, after hundreds of non-smooth
iterations, to ~1e-6 m in the mean with a handful of near-tie pixels (median /
L1-shrinkage branch flips) further out.
"""
import os

import numpy as np
import pytest

from oracle import oracle
from pdflow import scenes

# Oracle vs reference tolerances (FP32 restatement without FMA contraction).
FLOW_MEAN_TOL = 1e-5          # metres
FLOW_FRAC_OVER_1MM = 5e-4     # fraction of pixels allowed beyond 1e-3 m: near-tie branch
                              # flips of the FP32 reference itself (FP64 oracle: 13 of 76 800
                              # pixels at VGA rows=240)
FLOW_MAX_TOL = 2e-2           # metres (isolated branch flips)


def _frames(g):
    I1, Z1 = scenes.decode(g["i1"], g["z1"])
    I2, Z2 = scenes.decode(g["i2"], g["z2"])
    return I1, Z1, I2, Z2


def flow_stats(out, g, rows):
    st = {}
    for c, o in zip(("dx", "dy", "dz"), out):
        d = np.abs(o.astype(np.float64) - g[f"r{rows}_{c}"].astype(np.float64))
        st[c] = (d.mean(), d.max(), float((d > 1e-3).mean()))
    return st


CASES = [("qvga_s0.npz", 240, 320, 240), ("qvga_s0.npz", 60, 320, 240),
         ("vga_s2.npz", 480, 640, 480), ("vga_s2.npz", 240, 640, 480)]


@pytest.mark.parametrize("fixture,rows,w,h", CASES)
@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_oracle_flow_matches_reference(fixture, rows, w, h, precision):
    from conftest import load_golden
    g = load_golden(fixture)
    out = oracle.solve(rows, w, h, *_frames(g), precision=precision)
    for c, (mean, mx, frac) in flow_stats(out, g, rows).items():
        assert mean <= FLOW_MEAN_TOL, (c, mean)
        assert frac <= FLOW_FRAC_OVER_1MM, (c, frac)
        assert mx <= FLOW_MAX_TOL, (c, mx)


def test_golden_reference_was_repeatable(golden_qvga, golden_vga):
    for g, keys in ((golden_qvga, ("repeatable_r240", "repeatable_r60")),
                    (golden_vga, ("repeatable_r480", "repeatable_r240"))):
        for k in keys:
            assert bool(g[k]), k


def test_host_decode_is_the_reference_decode(golden_qvga):
    """uint16 * float(1/5000) and the column-major packing (scene_flow_impair.cpp:230-245)."""
    g = golden_qvga
    I, Z = oracle.decode_frame(g["i1"], g["z1"])
    I2, Z2 = scenes.decode(g["i1"], g["z1"])
    assert np.array_equal(I.view(np.uint32), I2.view(np.uint32))
    assert np.array_equal(Z.view(np.uint32), Z2.view(np.uint32))
    h, w = g["z1"].shape
    v, u = 17, 203
    assert Z[v + u * h] == np.float32(g["z1"][v, u]) * np.float32(1.0 / 5000.0)


SETUP_FIELDS = ("dct", "dcu", "dcv", "ddt", "ddu", "ddv", "mu", "ri", "rj", "ri_2", "rj_2", "sigma_pd",
                "sigma_puvx", "sigma_puvy", "sigma_pwx", "sigma_pwy", "tau_u", "tau_v", "tau_w")


def _max_rel_to_range(a, b):
    """max |a - b| relative to the field's range (max |b|)."""
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return float(np.abs(a - b).max() / (np.abs(b).max() + 1e-30))


@pytest.fixture(scope="module")
def oracle_r60_dumps(golden_qvga):
    _, _, _, st = oracle.solve(60, 320, 240, *_frames(golden_qvga), precision="f32", dump=True)
    return st


def test_oracle_pyramid_matches_reference(golden_qvga, oracle_r60_dumps):
    g, st = golden_qvga, oracle_r60_dumps
    for lv in (2, 3, 4):
        for fld in ("colour", "depth", "xx", "yy"):
            for frame, pre in (("old_push_", "pyr_old_"), ("push_", "pyr_new_")):
                ref = g[f"r60_{frame}{fld}_L{lv}"]
                ours = st[(pre + fld, lv)]
                assert np.allclose(ours, ref, rtol=2e-6, atol=4e-5), (fld, lv, frame)


@pytest.mark.parametrize("field", SETUP_FIELDS)
def test_oracle_level0_setup_matches_reference(golden_qvga, oracle_r60_dumps, field):
    """At the coarsest level both sides start from the same pyramid: the set-up
    stages agree to FP32 rounding."""
    ref = golden_qvga[f"r60_{field}_L0"]
    assert _max_rel_to_range(oracle_r60_dumps[(field, 0)], ref) <= 2e-5, field


@pytest.mark.parametrize("field", ("du_l", "dv_l", "dw_l", "du_prev", "dv_prev", "pd", "puu", "pwv", "sat_du"))
@pytest.mark.parametrize("level", (0, 1, 2))
def test_oracle_level_state_tracks_reference(golden_qvga, oracle_r60_dumps, field, level):
    key = f"r60_{field}_L{level}"
    if key not in golden_qvga.files:
        pytest.skip("not dumped")
    ref = golden_qvga[key]
    ours = oracle_r60_dumps[(field, level)]
    d = np.abs(ours.astype(np.float64) - ref)
    assert d.mean() <= 1e-4 * max(1.0, np.abs(ref).mean() * 100), (field, level, d.mean())


def test_median_sorting_network_sorts_every_zero_one_input():
    """The 9-input network of k_median (odd-even transposition: 9 rounds of
    neighbour exchanges (i, i+1), i of the round's parity, on a strict '<')
    sorts all 512 zero-one inputs, so by the 0-1 principle it sorts every
    input; on ties it keeps the input order, the stable order of the
    reference's bubble sort."""
    import itertools
    src = open(os.path.join(os.path.dirname(__file__), "..", "pd-flow_gb300", "csrc", "pdflow_kernels.cu")).read()
    assert "for (int r = 0; r < 9; ++r)" in src and "for (int a = r & 1; a + 1 < 9; a += 2)" in src
    assert "const bool sw_ = sf[a + 1] < sf[a];" in src
    net = [(a, a + 1) for r in range(9) for a in range(r & 1, 8, 2)]
    assert len(net) == 36
    for bits in itertools.product((0, 1), repeat=9):
        x = list(bits)
        for a, b in net:
            if x[b] < x[a]:
                x[a], x[b] = x[b], x[a]
        assert x == sorted(x)
    # stable: with strict exchanges equal values keep their input order
    rng = np.random.default_rng(0)
    for _ in range(500):
        vals = rng.integers(0, 3, size=9).astype(float)
        order = list(range(9))
        for a, b in net:
            if vals[order[b]] < vals[order[a]]:
                order[a], order[b] = order[b], order[a]
        assert order == sorted(range(9), key=lambda i: (vals[i], i))


def test_live_app_rgb_decode_every_value():
    """The oracle's RGB888 + millimetre conversion equals a numpy restatement of
    scene_flow_visualization.cpp:320-321 for every RGB triple and every depth
    value, and the 180-degree storage order of its camera loop."""
    k = np.arange(1 << 24, dtype=np.uint32)
    rgb = np.stack([k & 255, (k >> 8) & 255, k >> 16], axis=-1).astype(np.uint8).reshape(4096, 4096, 3)
    mm = (k & 0xFFFF).astype(np.uint16).reshape(4096, 4096)
    I, Z = oracle.decode_frame_rgb8_mm(rgb, mm, False)
    c = rgb.astype(np.float64)
    gray = ((0.299 * c[..., 0] + 0.587 * c[..., 1]) + 0.114 * c[..., 2]).astype(np.float32)
    depth = np.float32(0.001) * mm.astype(np.float32)
    assert np.array_equal(I.view(np.uint32), gray.T.ravel().view(np.uint32))
    assert np.array_equal(Z.view(np.uint32), depth.T.ravel().view(np.uint32))
    # hand-checked values: white stays 255, 1000 mm is 1 m
    assert I[0] == 0.0 and gray[4095, 4095] == np.float32(255.0) and depth[0, 1000] == np.float32(1.0)
    small = rgb[:5, :7]
    I0, Z0 = oracle.decode_frame_rgb8_mm(small, mm[:5, :7], False)
    I1, Z1 = oracle.decode_frame_rgb8_mm(small, mm[:5, :7], True)
    assert np.array_equal(I1.reshape(7, 5), I0.reshape(7, 5)[::-1, ::-1])
    assert np.array_equal(Z1.reshape(7, 5), Z0.reshape(7, 5)[::-1, ::-1])
