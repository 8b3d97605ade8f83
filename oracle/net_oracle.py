"""CPU oracle of the warm-start network (test infrastructure only).

A numpy restatement of the encoder-decoder the GPU library trains and runs
(pd-flow_gb300/csrc/pdflow_net.cu): same parameter layout, same layer order,
same input normalisation and loss.  With `quantize=True` it rounds to bfloat16
exactly where the GPU stores bfloat16 (weights, input, hidden activations,
pooled activations, back-propagated layer gradients) and accumulates in
float64, so GPU and oracle differ only by the GPU's FP32 accumulation order;
with `quantize=False` everything is float64, which is what the finite-
difference gradient check uses.

The reference has no learned component: this oracle pins the library's own
network, and its gradients are pinned against central finite differences.
"""
from __future__ import annotations

import numpy as np

H, W, HW = 80, 60, 4800
W_SCALE = 20.0

# (src1, up1, src2, cout, cout_pad, level, relu) in network order; activations
# are named by index: 0 = input, then one per conv/pool in creation order.
LEVELS = {0: (80, 60), 1: (40, 30), 2: (20, 15), 3: (10, 8)}


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    nan = np.isnan(a)
    if nan.any():
        out = out.copy()
        out[nan] = np.nan
    return out.reshape(a.shape)


class _Graph:
    def __init__(self):
        self.acts = []          # (C, H, W)
        self.convs = []         # dicts
        self.pools = []         # (in, out)
        x0 = self._act(8, 0)
        e1a = self._conv(x0, 0, -1, 16, 16, 0, 1)
        e1b = self._conv(e1a, 0, -1, 16, 16, 0, 1)
        p1 = self._pool(e1b, 1)
        e2a = self._conv(p1, 0, -1, 32, 32, 1, 1)
        e2b = self._conv(e2a, 0, -1, 32, 32, 1, 1)
        p2 = self._pool(e2b, 2)
        e3a = self._conv(p2, 0, -1, 64, 64, 2, 1)
        e3b = self._conv(e3a, 0, -1, 64, 64, 2, 1)
        p3 = self._pool(e3b, 3)
        e4a = self._conv(p3, 0, -1, 96, 96, 3, 1)
        e4b = self._conv(e4a, 0, -1, 96, 96, 3, 1)
        d3 = self._conv(e4b, 1, e3b, 64, 64, 2, 1)
        d2 = self._conv(d3, 1, e2b, 32, 32, 1, 1)
        d1 = self._conv(d2, 1, e1b, 16, 16, 0, 1)
        self._conv(d1, 0, -1, 3, 16, 0, 0)
        off = 0
        for c in self.convs:
            c["woff"] = off
            off += c["cout"] * c["K"]
            c["boff"] = off
            off += c["cout"]
        self.nparams = off

    def _act(self, C, level):
        self.acts.append((C,) + LEVELS[level])
        return len(self.acts) - 1

    def _conv(self, s1, up1, s2, cout, cout_pad, level, relu):
        c1 = self.acts[s1][0]
        c2 = self.acts[s2][0] if s2 >= 0 else 0
        out = self._act(cout_pad, level)
        self.convs.append(dict(src1=s1, up1=up1, src2=s2, c1=c1, c2=c2, cout=cout, cout_pad=cout_pad,
                               level=level, relu=relu, out=out, K=9 * (c1 + c2)))
        return out

    def _pool(self, a, level):
        out = self._act(self.acts[a][0], level)
        self.pools.append((a, out))
        return out


GRAPH = _Graph()
POOL_AFTER = (1, 3, 5)      # conv indices whose output is pooled


def param_count() -> int:
    return GRAPH.nparams


def _im2col(x):
    """x [n, H, W, C] -> [n*H*W, 9*C] (tap-major, zero padding)."""
    n, h, w, c = x.shape
    xp = np.zeros((n, h + 2, w + 2, c), x.dtype)
    xp[:, 1:-1, 1:-1] = x
    cols = [xp[:, dh:dh + h, dw:dw + w] for dh in range(3) for dw in range(3)]
    return np.stack(cols, axis=3).reshape(n * h * w, 9 * c)


def _col2im(dcol, n, h, w, c):
    """Adjoint of _im2col: [n*H*W, 9*C] -> [n, H, W, C]."""
    d = dcol.reshape(n, h, w, 9, c)
    out = np.zeros((n, h + 2, w + 2, c), dcol.dtype)
    for t in range(9):
        dh, dw = t // 3, t % 3
        out[:, dh:dh + h, dw:dw + w] += d[:, :, :, t]
    return out[:, 1:-1, 1:-1]


def _up(x, h, w):
    return x.repeat(2, axis=1).repeat(2, axis=2)[:, :h, :w]


def _up_grad(g, h1, w1):
    n, h, w, c = g.shape
    gp = np.zeros((n, 2 * h1, 2 * w1, c), g.dtype)
    gp[:, :h, :w] = g
    return gp.reshape(n, h1, 2, w1, 2, c).sum(axis=(2, 4))


def _pool(x):
    n, h, w, c = x.shape
    ho, wo = (h + 1) // 2, (w + 1) // 2
    xp = np.zeros((n, 2 * ho, 2 * wo, c), np.float64)
    cnt = np.zeros((1, 2 * ho, 2 * wo, 1))
    xp[:, :h, :w] = x
    cnt[:, :h, :w] = 1
    s = xp.reshape(n, ho, 2, wo, 2, c).sum(axis=(2, 4))
    k = cnt.reshape(1, ho, 2, wo, 2, 1).sum(axis=(2, 4))
    return s / k, k


def normalise_input(inp):
    """inp [n, 4, 4800] (I1, I2, Z1, Z2) -> [n, 80, 60, 8] float (unrounded)."""
    inp = np.asarray(inp, np.float32).reshape(-1, 4, HW)
    n = inp.shape[0]
    x = np.zeros((n, HW, 8), np.float32)
    x[:, :, 0] = inp[:, 0] * np.float32(1 / 255) - np.float32(0.5)
    x[:, :, 1] = inp[:, 1] * np.float32(1 / 255) - np.float32(0.5)
    for k, z in ((2, inp[:, 2]), (3, inp[:, 3])):
        x[:, :, k] = np.where(z > 0, np.float32(0.5) * (z - np.float32(2.5)), np.float32(-1.5))
    return x.reshape(n, H, W, 8)


class NetOracle:
    def __init__(self, params, quantize: bool = True):
        self.p = np.asarray(params, np.float64)
        assert self.p.size == GRAPH.nparams
        self.q = quantize

    def _r(self, x):
        return bf16(x).astype(np.float64) if self.q else np.asarray(x, np.float64)

    def weights(self, i):
        c = GRAPH.convs[i]
        w = self.p[c["woff"]:c["woff"] + c["cout"] * c["K"]].reshape(c["cout"], c["K"])
        b = self.p[c["boff"]:c["boff"] + c["cout"]]
        return self._r(w.astype(np.float32)) if self.q else w, b

    def _conv_input(self, acts, c):
        n = acts[0].shape[0]
        h, w = LEVELS[c["level"]]
        a1 = acts[c["src1"]]
        if c["up1"]:
            a1 = _up(a1, h, w)
        x = a1 if c["src2"] < 0 else np.concatenate([a1, acts[c["src2"]]], axis=3)
        return x, n, h, w

    def forward(self, inp):
        """Returns (head output [n*4800, 3] with dw scaled by 20, cache)."""
        x0 = self._r(normalise_input(inp))
        acts = [None] * len(GRAPH.acts)
        acts[0] = x0
        cols = []
        pre = []
        pi = 0
        for i, c in enumerate(GRAPH.convs):
            x, n, h, w = self._conv_input(acts, c)
            col = _im2col(x)
            wq, b = self.weights(i)
            y = col @ wq.T + b[None, :]
            cols.append(col)
            if c["relu"]:
                y = np.maximum(y, 0.0)
                acts[c["out"]] = self._r(y.astype(np.float32) if self.q else y).reshape(n, h, w, c["cout_pad"])
            else:
                acts[c["out"]] = y.reshape(n, h, w, c["cout"])
            pre.append(y)
            if pi < 3 and i == POOL_AFTER[pi]:
                a, o = GRAPH.pools[pi]
                pooled, _ = _pool(acts[a])
                acts[o] = self._r(pooled.astype(np.float32)) if self.q else pooled
                pi += 1
        head = acts[GRAPH.convs[-1]["out"]].reshape(-1, 3)
        return head, dict(acts=acts, cols=cols)

    def predict(self, inp):
        head, _ = self.forward(inp)
        n = head.shape[0] // HW
        out = head.reshape(n, HW, 3).transpose(0, 2, 1).copy()
        out[:, 2] /= W_SCALE
        return out

    def loss_and_grads(self, inp, label):
        """Masked MSE against label [n, 3, 4800] (du, dv, dw) and the gradient
        w.r.t. every parameter (the library's parameter layout)."""
        inp = np.asarray(inp, np.float32).reshape(-1, 4, HW)
        n = inp.shape[0]
        head, cache = self.forward(inp)
        acts, cols = cache["acts"], cache["cols"]
        t = np.asarray(label, np.float64).reshape(n, 3, HW).transpose(0, 2, 1).reshape(-1, 3).copy()
        t[:, 2] *= W_SCALE
        valid = (inp[:, 2] > 0).reshape(-1)
        cnt = int(valid.sum())
        d = (head - t) * valid[:, None]
        loss = float((d * d).sum() / (3 * cnt))
        dout = 2.0 * d / (3 * cnt)
        if self.q:
            dout = dout.astype(np.float32).astype(np.float64)
        grads = np.zeros(GRAPH.nparams)
        gacts = [np.zeros(a.shape) if a is not None else None for a in acts]
        gy = None
        for i in range(len(GRAPH.convs) - 1, -1, -1):
            c = GRAPH.convs[i]
            for q in range(3):
                if POOL_AFTER[q] == i:
                    a, o = GRAPH.pools[q]
                    _, k = _pool(acts[a])
                    g = (gacts[o] / k)
                    h, w = acts[a].shape[1:3]
                    gacts[a] += g.repeat(2, axis=1).repeat(2, axis=2)[:, :h, :w]
            if c["relu"]:
                gy = gacts[c["out"]].reshape(-1, c["cout_pad"]) * (acts[c["out"]].reshape(-1, c["cout_pad"]) > 0)
            else:
                gy = dout
            gy = self._r(gy.astype(np.float32)) if self.q else gy
            col = cols[i]
            grads[c["woff"]:c["woff"] + c["cout"] * c["K"]] = (gy.T @ col).reshape(-1)
            grads[c["boff"]:c["boff"] + c["cout"]] = gy.sum(axis=0)
            if i == 0:
                break
            wq, _ = self.weights(i)
            dcol = gy @ wq
            h, w = LEVELS[c["level"]]
            dx = _col2im(dcol, n, h, w, c["c1"] + c["c2"])
            d1 = dx[..., :c["c1"]]
            if c["up1"]:
                h1, w1 = acts[c["src1"]].shape[1:3]
                d1 = _up_grad(d1, h1, w1)
            gacts[c["src1"]] += d1
            if c["src2"] >= 0:
                gacts[c["src2"]] += dx[..., c["c1"]:]
        return loss, grads


def init_params(seed: int = 1):
    """Random He-normal parameters (numpy RNG; not the library's initialiser)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(GRAPH.nparams, np.float32)
    for i, c in enumerate(GRAPH.convs):
        cin = c["c1"] + c["c2"]
        used = 4 if i == 0 else cin
        w = rng.normal(size=(c["cout"], 9, cin)) * np.sqrt(2.0 / (9 * used)) * (1.0 if c["relu"] else 0.1)
        if i == 0:
            w[:, :, 4:] = 0
        p[c["woff"]:c["woff"] + c["cout"] * c["K"]] = w.reshape(-1)
        p[c["boff"]:c["boff"] + c["cout"]] = rng.normal(size=c["cout"]) * 0.01
    return p
