"""The tcgen05 BF16 GEMM and the warm-start network's forward and backward
kernels against the CPU oracle (oracle/net_oracle.py)."""
import numpy as np
import pytest

from oracle import net_oracle as no
from pdflow import Net, gemm_bf16

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch(built_lib):
    return pytest.importorskip("torch")


def bf16_tensor(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().to(torch.bfloat16)


@pytest.mark.parametrize("M,N,K,kps", [(128, 16, 64, 0), (1000, 128, 72, 0), (257, 96, 1440, 0), (300, 200, 200, 0),
                                       (96, 16, 4096, 512), (5, 48, 8, 0)])
def test_gemm_matches_float64_product_of_bf16_operands(torch, M, N, K, kps):
    rng = np.random.default_rng(M * 7 + N + K)
    A = no.bf16(rng.normal(size=(M, K)))
    B = no.bf16(rng.normal(size=(N, K)))
    dA, dB = bf16_tensor(torch, A), bf16_tensor(torch, B)
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    gemm_bf16(M, N, K, dA.data_ptr(), K, dB.data_ptr(), K, C.data_ptr(), N, kps)
    got = C.cpu().numpy().astype(np.float64)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64).T
    assert np.all(np.abs(got - ref) <= 1e-6 * scale + 1e-30), np.abs(got - ref).max()


def _batch(seed, n):
    rng = np.random.default_rng(seed)
    inp = np.zeros((n, 4, no.HW), np.float32)
    inp[:, 0:2] = rng.uniform(0, 255, size=(n, 2, no.HW))
    inp[:, 2:4] = rng.uniform(0.8, 4.0, size=(n, 2, no.HW))
    inp[:, 2][rng.random((n, no.HW)) < 0.05] = 0
    label = (rng.normal(size=(n, 3, no.HW)) * np.array([1, 1, 0.02])[None, :, None]).astype(np.float32)
    return inp, label


def test_forward_matches_oracle(torch):
    n = 3
    net = Net(4, seed=7)
    p = no.init_params(11)
    net.set_params(p)
    assert np.array_equal(net.get_params(), p)
    inp, _ = _batch(1, n)
    d_in = torch.from_numpy(inp).cuda()
    d_out = torch.zeros((n, 3, no.HW), dtype=torch.float32, device="cuda")
    net.forward(n, d_in.data_ptr(), d_out.data_ptr())
    got = d_out.cpu().numpy()
    ref = no.NetOracle(p, quantize=True).predict(inp)
    err = np.abs(got - ref)
    for c in range(3):     # bf16 roundings that land on the other side of a tie propagate: tolerance per channel
        s = np.abs(ref[:, c]).max()
        assert err[:, c].max() <= 2e-2 * s and err[:, c].mean() <= 1e-3 * s, (c, err[:, c].max(), s)
    net.close()


def test_gathered_convolutions_equal_the_im2col_ones(torch):
    """From 16 inputs on the convolution GEMMs gather their im2col operand while
    staging it; below 16 a separate im2col kernel builds it.  Each output row
    of a GEMM accumulates the same products in the same order either way, so
    20 inputs in one forward equal the same inputs in forwards of 4, bit for bit."""
    n, chunk = 20, 4
    net = Net(n, seed=3)
    net.set_params(no.init_params(5))
    inp, _ = _batch(2, n)
    d_in = torch.from_numpy(inp).cuda()
    whole = torch.zeros((n, 3, no.HW), dtype=torch.float32, device="cuda")
    net.forward(n, d_in.data_ptr(), whole.data_ptr())
    parts = torch.zeros((n, 3, no.HW), dtype=torch.float32, device="cuda")
    for k in range(0, n, chunk):
        net.forward(chunk, d_in[k:k + chunk].data_ptr(), parts[k:k + chunk].data_ptr())
    torch.cuda.synchronize()
    net.close()
    assert np.array_equal(whole.cpu().numpy().view(np.uint32), parts.cpu().numpy().view(np.uint32))


def test_gradients_match_oracle(torch):
    """GPU gradients against the oracle with the same bf16 rounding points.  The
    GPU's FP32 accumulation flips some bf16 roundings, so the tolerance is
    tied to how far bf16 rounding itself moves the gradient (the quantised
    oracle against the float64 one): the GPU must stay well inside it."""
    n = 2
    net = Net(2, seed=3)
    p = no.init_params(12)
    net.set_params(p)
    inp, label = _batch(2, n)
    d_in = torch.from_numpy(inp).cuda()
    d_lab = torch.from_numpy(label).cuda()
    loss, g = net.gradients(n, d_in.data_ptr(), d_lab.data_ptr())
    rloss, rq = no.NetOracle(p, quantize=True).loss_and_grads(inp, label)
    _, rf = no.NetOracle(p, quantize=False).loss_and_grads(inp, label)
    assert abs(loss - rloss) <= 1e-5 * rloss
    rel = lambda x, y: np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-30)
    for i, c in enumerate(no.GRAPH.convs):
        for lo, hi in ((c["woff"], c["woff"] + c["cout"] * c["K"]), (c["boff"], c["boff"] + c["cout"])):
            a, q, f = g[lo:hi].astype(np.float64), rq[lo:hi], rf[lo:hi]
            e_gpu, e_bf16 = rel(a, q), rel(q, f)
            assert e_gpu <= 0.75 * e_bf16 + 2e-3 and e_gpu <= 0.05, (i, lo, e_gpu, e_bf16)
            cos = float(a @ f / max(np.linalg.norm(a) * np.linalg.norm(f), 1e-30))
            assert cos >= 0.99, (i, lo, cos)
    net.close()


def test_training_steps_reduce_the_loss(torch):
    """A target the network can represent (a pointwise function of its
    inputs) is learned: the loss falls well below the zero prediction's."""
    n = 4
    net = Net(n, seed=5)
    inp, _ = _batch(3, n)
    z1 = inp[:, 2]
    label = np.stack([inp[:, 0] / 255.0 - 0.5, np.where(z1 > 0, 0.5 * (z1 - 2.5), 0.0),
                      0.02 * (inp[:, 1] / 255.0 - 0.5)], axis=1).astype(np.float32)
    d_in = torch.from_numpy(inp).cuda()
    d_lab = torch.from_numpy(label).cuda()
    losses = [net.train_step(n, d_in.data_ptr(), d_lab.data_ptr(), 2e-3) for _ in range(60)]
    assert all(np.isfinite(losses))
    assert losses[-1] < 0.3 * losses[0], losses[::10]
    net.close()
