"""The warm-start network's CPU oracle: its gradients against central finite
differences (float64, no bfloat16 rounding), and its bf16 rounding."""
import numpy as np
import pytest

from oracle import net_oracle as no


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 3.0e38, 1e-40], np.float32)
    r = no.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # tie -> even
    assert r[2] == np.float32(1.0 + 4 * 2 ** -8)   # tie -> even (up)
    assert r[3] == -2.5 and r[4] == 0.0
    assert np.all(r.view(np.uint32) & 0xFFFF == 0)


def test_parameter_count_is_about_a_third_of_a_million():
    assert 300_000 < no.param_count() < 400_000


def _batch(seed, n=1):
    rng = np.random.default_rng(seed)
    inp = np.zeros((n, 4, no.HW), np.float32)
    inp[:, 0:2] = rng.uniform(0, 255, size=(n, 2, no.HW))
    inp[:, 2:4] = rng.uniform(0.8, 4.0, size=(n, 2, no.HW))
    inp[:, 2][rng.random((n, no.HW)) < 0.05] = 0
    label = rng.normal(size=(n, 3, no.HW)).astype(np.float32) * np.array([1, 1, 0.02], np.float32)[None, :, None]
    return inp, label


def test_gradients_match_central_differences():
    p = no.init_params(3).astype(np.float64)
    inp, label = _batch(5)
    net = no.NetOracle(p, quantize=False)
    loss, g = net.loss_and_grads(inp, label)
    rng = np.random.default_rng(9)
    idx = []
    for c in no.GRAPH.convs:               # a few weights and one bias of every layer
        w = rng.integers(c["woff"], c["woff"] + c["cout"] * c["K"], size=2)
        idx += list(w) + [c["boff"] + int(rng.integers(0, c["cout"]))]
    eps = 1e-6                              # small enough not to cross ReLU kinks
    for i in idx:
        if i < no.GRAPH.convs[0]["boff"] and (i - no.GRAPH.convs[0]["woff"]) % 8 >= 4:
            continue                        # padding input channels: no effect
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        lp, _ = no.NetOracle(pp, quantize=False).loss_and_grads(inp, label)
        lm, _ = no.NetOracle(pm, quantize=False).loss_and_grads(inp, label)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-3 * abs(fd) + 1e-10, (i, fd, g[i])


def test_quantized_forward_stays_close_to_float64():
    p = no.init_params(4)
    inp, _ = _batch(6, n=2)
    a = no.NetOracle(p, quantize=True).predict(inp)
    b = no.NetOracle(p, quantize=False).predict(inp)
    assert np.abs(a - b).max() <= 0.05 * np.abs(b).max()
