"""Evaluates the learned warm start against the plain solver on held-out pairs.

    python -m pdflow.eval_warmstart --weights warmstart.npz --rows 480 --pairs 64 --scales 0.5

For each iteration scale it solves the same batch several ways and reports,
per way, the end-point error against the plain result and against the
scenes' ground-truth motion (metres, mean over pixels with valid frame-1
depth, then mean / max over pairs), the final energy relative to the plain
solve's, and the time of the batch:

* plain      the reference schedule (pdflow_solve_batch);
* learned    pdflow_solve_batch_learned (network seed at 60x80, scaled
             iterations, energy fallback);
* zero-seed  the same schedule started at 60x80 from zero flow (the learned
             path without its network);
* scaled     the plain schedule from the coarsest level with every level's
             iterations scaled (the same iteration budget without a seed);
* label_seed the scaled schedule from 60x80 seeded with the plain result
             itself averaged to 60x80 (what a perfect network would predict).

`--schedules "25,40,55,70,85,95;..."` also solves the batch with plain
schedules of other per-level iteration counts (coarsest level first) and
reports their end-point error against the reference schedule's result and
their time: how far a trajectory change moves the non-converged result.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import BatchSolver, Net, datagen

HW = 4800


def epe(a, b, valid):
    d = np.sqrt((a[0] - b[0]) ** 2 + (a[1] - b[1]) ** 2 + (a[2] - b[2]) ** 2)
    return np.array([d[k][valid[k]].mean() for k in range(d.shape[0])])


def load_weights(path: str) -> np.ndarray:
    with np.load(path) as f:
        return np.asarray(f["params"], np.float32)


def evaluate(weights, rows: int, pairs: int, scales, seed0: int = 3_000_000, margin: float = 0.01, log=print):
    import torch

    vga = rows == 480
    w, h = (640, 480) if vga else (320, 240)
    dev = torch.device("cuda")
    rng = np.random.default_rng(seed0)
    seeds = list(range(seed0, seed0 + pairs))
    nobj = {s: int(rng.integers(1, 9)) for s in seeds}
    i1, z1, i2, z2, gt = datagen.render_pairs(torch, seeds, vga, n_objects=lambda s: nobj[s], with_flow=True)
    valid = (z1.cpu().numpy().view(np.uint16) > 0).transpose(0, 2, 1).reshape(pairs, -1)
    gt = gt.cpu().numpy()
    gt = [gt[:, 0], gt[:, 1], gt[:, 2]]
    if rows != h:
        raise ValueError("rows must equal the image height (240 for QVGA, 480 for VGA)")
    net = Net(pairs, seed=1)
    net.set_params(weights)
    b = BatchSolver(rows, w, h, pairs)

    def push():
        b.push_raw_device(pairs, i1.data_ptr(), z1.data_ptr())
        b.push_raw_device(pairs, i2.data_ptr(), z2.data_ptr())

    def timed(fn, reps=3):
        fn()
        b.synchronize()
        best = float("inf")
        for _ in range(reps):
            t = time.perf_counter()
            r = fn()
            b.synchronize()
            best = min(best, time.perf_counter() - t)
        return r, best

    push()
    _, t_plain = timed(lambda: b.solve(pairs))
    plain = b.read_flow(pairs)
    e_plain = b.energy(pairs)
    label = torch.zeros((pairs, 3, HW), dtype=torch.float32, device=dev)
    b.seed_level_labels(pairs, label.data_ptr())
    ep_gt_plain = epe(plain, gt, valid)
    out = dict(rows=rows, pairs=pairs, plain_ms=t_plain * 1e3, plain_pairs_s=pairs / t_plain,
               plain_epe_gt_m=float(ep_gt_plain.mean()), scales={})
    zero_seed = torch.zeros((pairs, 3, HW), dtype=torch.float32, device=dev)
    for s in scales:
        rep, t_l = timed(lambda: b.solve_learned(pairs, net, s, margin))
        learned = b.read_flow(pairs)
        e_l = b.energy(pairs)
        ep_l = epe(learned, plain, valid)
        b.solve_levels(pairs, 2, 99, zero_seed.data_ptr(), s)
        zs = b.read_flow(pairs)
        e_z = b.energy(pairs)
        b.solve_levels(pairs, 0, 99, None, s)
        sc = b.read_flow(pairs)
        e_s = b.energy(pairs)
        b.solve_levels(pairs, 2, 99, label.data_ptr(), s)
        ls = b.read_flow(pairs)
        e_ls = b.energy(pairs)
        r = dict(learned_ms=t_l * 1e3, learned_pairs_s=pairs / t_l, fallbacks=rep["fallbacks"],
                 max_seed_energy_ratio=rep["max_energy_ratio"])
        for name, flow, en in (("learned", learned, e_l), ("zero_seed", zs, e_z), ("scaled", sc, e_s),
                               ("label_seed", ls, e_ls)):
            ep = ep_l if name == "learned" else epe(flow, plain, valid)
            r[name] = dict(epe_mean_m=float(ep.mean()), epe_max_pair_m=float(ep.max()),
                           epe_gt_mean_m=float(epe(flow, gt, valid).mean()),
                           energy_ratio_mean=float((en / e_plain).mean()), energy_ratio_max=float((en / e_plain).max()))
        out["scales"][str(s)] = r
        log(json.dumps({str(s): r}))
    b.close()
    net.close()
    return out


def schedule_sweep(schedules, rows: int, pairs: int, seed0: int = 3_000_000, log=print):
    """The plain batch under other per-level iteration counts, against the
    reference schedule's result (same held-out pairs as `evaluate`)."""
    import torch

    from . import _lib
    vga = rows == 480
    w, h = (640, 480) if vga else (320, 240)
    rng = np.random.default_rng(seed0)
    seeds = list(range(seed0, seed0 + pairs))
    nobj = {s: int(rng.integers(1, 9)) for s in seeds}
    i1, z1, i2, z2, gt = datagen.render_pairs(torch, seeds, vga, n_objects=lambda s: nobj[s], with_flow=True)
    valid = (z1.cpu().numpy().view(np.uint16) > 0).transpose(0, 2, 1).reshape(pairs, -1)
    gt = gt.cpu().numpy()
    gt = [gt[:, 0], gt[:, 1], gt[:, 2]]

    def run(iters):
        p = _lib.default_params(rows)
        for k, v in enumerate(iters):
            p.num_max_iter[k] = v
        b = BatchSolver(rows, w, h, pairs, params=p)
        b.push_raw_device(pairs, i1.data_ptr(), z1.data_ptr())
        b.push_raw_device(pairs, i2.data_ptr(), z2.data_ptr())
        b.autotune(pairs)
        b.solve(pairs)
        b.synchronize()
        best = float("inf")
        for _ in range(3):
            t = time.perf_counter()
            b.solve(pairs)
            b.synchronize()
            best = min(best, time.perf_counter() - t)
        out = b.read_flow(pairs)
        b.close()
        return out, best

    p0 = _lib.default_params(rows)
    levels = (rows // 15).bit_length()
    ref_iters = [p0.num_max_iter[k] for k in range(levels)]
    ref, t0 = run(ref_iters)
    res = [dict(schedule=ref_iters, ms=t0 * 1e3, epe_gt_mm=float(epe(ref, gt, valid).mean() * 1e3))]
    log(json.dumps(res[0]))
    for it in schedules:
        out, t = run(it)
        e = epe(out, ref, valid)
        r = dict(schedule=it, ms=t * 1e3, speedup=t0 / t, epe_vs_plain_mm=float(e.mean() * 1e3),
                 epe_vs_plain_max_pair_mm=float(e.max() * 1e3), epe_gt_mm=float(epe(out, gt, valid).mean() * 1e3))
        res.append(r)
        log(json.dumps(r))
    return res


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--weights", required=True)
    ap.add_argument("--rows", type=int, default=480, choices=(240, 480))
    ap.add_argument("--pairs", type=int, default=64)
    ap.add_argument("--scales", default="0.5")
    ap.add_argument("--margin", type=float, default=0.01)
    ap.add_argument("--schedules", default="",
                    help="plain schedules to compare, e.g. \"25,40,55,70,85,95;25,40,55,70,43,100\"")
    a = ap.parse_args()
    if a.schedules:
        schedule_sweep([[int(x) for x in s.split(",")] for s in a.schedules.split(";") if s], a.rows, a.pairs)
    res = evaluate(load_weights(a.weights), a.rows, a.pairs, [float(x) for x in a.scales.split(",")],
                   margin=a.margin)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
