"""The learned warm start with the shipped weights: accuracy against the
scenes' ground-truth motion and energy against the plain solver, what the
network gains over the same schedule without it, and the fallback rule."""
import numpy as np
import pytest

from oracle import net_oracle as no
from pdflow import BatchSolver, Net, datagen, load_weights

pytestmark = pytest.mark.gpu

PAIRS = 12


def epe(a, b, valid):
    d = np.sqrt(sum((x - y) ** 2 for x, y in zip(a, b)))
    return np.array([d[k][valid[k]].mean() for k in range(d.shape[0])])


@pytest.fixture(scope="module")
def vga_batch(built_lib):
    torch = pytest.importorskip("torch")
    seeds = list(range(7_000_000, 7_000_000 + PAIRS))
    rng = np.random.default_rng(1)
    nobj = {s: int(rng.integers(1, 9)) for s in seeds}
    i1, z1, i2, z2, gt = datagen.render_pairs(torch, seeds, True, n_objects=lambda s: nobj[s], with_flow=True)
    valid = (z1.cpu().numpy().view(np.uint16) > 0).transpose(0, 2, 1).reshape(PAIRS, -1)
    g = gt.cpu().numpy()
    b = BatchSolver(480, 640, 480, PAIRS)
    b.push_raw_device(PAIRS, i1.data_ptr(), z1.data_ptr())
    b.push_raw_device(PAIRS, i2.data_ptr(), z2.data_ptr())
    b.solve(PAIRS)
    plain = b.read_flow(PAIRS)
    e_plain = b.energy(PAIRS)
    yield dict(torch=torch, b=b, valid=valid, gt=[g[:, 0], g[:, 1], g[:, 2]], plain=plain, e_plain=e_plain)
    b.close()


def test_learned_full_iterations_beat_plain_against_ground_truth(vga_batch):
    d = vga_batch
    net = Net(PAIRS)
    net.set_params(load_weights())
    rep = d["b"].solve_learned(PAIRS, net, iter_scale=1.0, energy_margin=-1.0)
    learned = d["b"].read_flow(PAIRS)
    e = d["b"].energy(PAIRS)
    net.close()
    assert rep["fallbacks"] == 0
    gt_plain = epe(d["plain"], d["gt"], d["valid"]).mean()
    gt_learned = epe(learned, d["gt"], d["valid"]).mean()
    assert gt_learned < gt_plain                      # closer to the true motion
    assert (e / d["e_plain"]).mean() < 1.0            # lower energy of the same functional
    # ~1.1 mm: the seed replaces the plain 60x80 state and so changes the
    # trajectory of the non-converged fixed-count iterations (see the next test)
    assert epe(learned, d["plain"], d["valid"]).mean() < 2e-3


def test_plain_result_moves_with_its_own_iteration_count(vga_batch):
    """The scale of the "1 mm against plain" bar: the plain schedule with
    five fewer iterations at the finest level (95 instead of 100) already lands
    about 1 mm from the plain result, because the reference's fixed iteration
    counts stop far from convergence.  A warm start that changes the
    trajectory cannot stay within that bar."""
    d = vga_batch
    from pdflow import _lib
    p = _lib.default_params(480)
    p.num_max_iter[5] = 95
    torch = d["torch"]
    seeds = list(range(7_000_000, 7_000_000 + PAIRS))
    rng = np.random.default_rng(1)
    nobj = {s: int(rng.integers(1, 9)) for s in seeds}
    i1, z1, i2, z2 = datagen.render_pairs(torch, seeds, True, n_objects=lambda s: nobj[s])
    b = BatchSolver(480, 640, 480, PAIRS, params=p)
    b.push_raw_device(PAIRS, i1.data_ptr(), z1.data_ptr())
    b.push_raw_device(PAIRS, i2.data_ptr(), z2.data_ptr())
    b.solve(PAIRS)
    fewer = b.read_flow(PAIRS)
    b.close()
    moved = epe(fewer, d["plain"], d["valid"]).mean()
    assert 3e-4 < moved < 3e-3, moved


def test_network_gains_over_the_same_schedule_without_it(vga_batch):
    d = vga_batch
    torch = d["torch"]
    net = Net(PAIRS)
    net.set_params(load_weights())
    d["b"].solve_learned(PAIRS, net, iter_scale=0.75, energy_margin=-1.0)
    learned = d["b"].read_flow(PAIRS)
    e_l = d["b"].energy(PAIRS)
    net.close()
    zero = torch.zeros((PAIRS, 3, 4800), dtype=torch.float32, device="cuda")
    d["b"].solve_levels(PAIRS, 2, 99, zero.data_ptr(), 0.75)
    zs = d["b"].read_flow(PAIRS)
    e_z = d["b"].energy(PAIRS)
    d["b"].solve_levels(PAIRS, 0, 99, None, 0.75)
    sc = d["b"].read_flow(PAIRS)
    gt = lambda f: epe(f, d["gt"], d["valid"]).mean()
    assert gt(learned) < gt(zs) and gt(learned) < gt(sc)
    assert e_l.mean() < e_z.mean()


def test_fallback_pairs_equal_the_plain_solve(vga_batch):
    d = vga_batch
    net = Net(PAIRS)
    net.set_params(no.init_params(3) * 0.0)            # predicts zero flow: a poor seed
    rep = d["b"].solve_learned(PAIRS, net, iter_scale=0.5, energy_margin=0.0)
    out = d["b"].read_flow(PAIRS)
    ep, el = d["b"].learned_energies(PAIRS)
    net.close()
    fell = el > ep
    assert rep["fallbacks"] == int(fell.sum()) > 0
    for k in np.nonzero(fell)[0]:
        for c in range(3):
            assert np.array_equal(out[c][k].view(np.uint32), d["plain"][c][k].view(np.uint32))


def test_accepted_and_rejected_pairs_in_one_batch(vga_batch):
    """With a margin that splits the batch, the accepted pairs equal the same
    learned solve without a fallback rule and the rejected ones equal the
    plain solve, bit for bit."""
    d = vga_batch
    net = Net(PAIRS)
    net.set_params(load_weights())
    for scale in (0.5, 0.25, 0.1):   # fewer iterations raise the learned energies
        d["b"].solve_learned(PAIRS, net, iter_scale=scale, energy_margin=-1.0)
        free = d["b"].read_flow(PAIRS)
        ep, el = d["b"].learned_energies(PAIRS)
        ratio = el / ep
        if ratio.max() > 1.0 and ratio.min() < ratio.max():
            break
    margin = float((ratio.max() + max(1.0, ratio.min())) / 2) - 1.0
    rep = d["b"].solve_learned(PAIRS, net, iter_scale=scale, energy_margin=margin)
    out = d["b"].read_flow(PAIRS)
    net.close()
    fell = ~(el <= np.float32(1.0 + np.float32(margin)) * ep)
    assert 0 < rep["fallbacks"] == int(fell.sum()) < PAIRS
    for k in range(PAIRS):
        ref = d["plain"] if fell[k] else free
        for c in range(3):
            assert np.array_equal(out[c][k].view(np.uint32), ref[c][k].view(np.uint32)), (k, c, bool(fell[k]))
