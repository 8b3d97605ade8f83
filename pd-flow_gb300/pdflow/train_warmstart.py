"""Trains the warm-start network on flows the plain solver produces.

    python -m pdflow.train_warmstart --pairs 20000 --epochs 12 --out weights.npz

1. renders `--pairs` seeded synthetic pairs on the GPU (half QVGA rows=240,
   half VGA rows=480; 1-8 moving objects; seeds from 1_000_000 up, disjoint
   from every test and benchmark seed);
2. solves them with the plain batched solver and keeps, per pair, the
   network's input (both frames' 60x80 level images) and its label (the
   plain final flow averaged down to the 60x80 level);
3. trains the network with the library's own tcgen05 forward/backward kernels
   and Adam (cosine learning-rate decay), holding out 5 % for validation;
4. writes the FP32 parameters and the training record to `--out`.

torch holds the device buffers; every render, solve, forward, backward and
update runs in libpdflow_gb300.so.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import BatchSolver, Net, datagen

HW = 4800


def build_dataset(torch, n_pairs: int, batch: int, log):
    dev = torch.device("cuda")
    n_half = n_pairs // 2
    inputs = torch.empty((n_pairs, 4, HW), dtype=torch.float32, device=dev)
    labels = torch.empty((n_pairs, 3, HW), dtype=torch.float32, device=dev)
    rng = np.random.default_rng(2024)
    k = 0
    t0 = time.time()
    for vga, rows, count in ((False, 240, n_half), (True, 480, n_pairs - n_half)):
        w, h = (640, 480) if vga else (320, 240)
        solver = BatchSolver(rows, w, h, batch)
        seed0 = 1_000_000 + (500_000 if vga else 0)
        done = 0
        while done < count:
            nb = min(batch, count - done)
            seeds = [seed0 + done + j for j in range(nb)]
            nobj = {s: int(rng.integers(1, 9)) for s in seeds}
            i1, z1, i2, z2 = datagen.render_pairs(torch, seeds, vga, n_objects=lambda s: nobj[s])
            solver.push_raw_device(nb, i1.data_ptr(), z1.data_ptr())
            solver.push_raw_device(nb, i2.data_ptr(), z2.data_ptr())
            solver.solve(nb)
            solver.synchronize()
            solver.seed_level_inputs(nb, inputs[k:k + nb].data_ptr())
            solver.seed_level_labels(nb, labels[k:k + nb].data_ptr())
            k += nb
            done += nb
        solver.close()
        log(f"dataset: {count} {'VGA' if vga else 'QVGA'} pairs solved ({time.time() - t0:.1f} s)")
    return inputs, labels


def masked_mse(torch, pred, label, inp):
    valid = (inp[:, 2] > 0).unsqueeze(1).float()
    scale = torch.tensor([1.0, 1.0, 20.0], device=pred.device).view(1, 3, 1)
    d = (pred - label) * scale * valid
    return float((d * d).sum() / (3.0 * valid.sum()))


def train(args, log=print):
    import torch

    t_start = time.time()
    inputs, labels = build_dataset(torch, args.pairs, args.batch, log)
    n = inputs.shape[0]
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    perm = torch.randperm(n, generator=g, device="cuda")
    n_val = max(args.batch, n // 20)
    val_idx, train_idx = perm[:n_val], perm[n_val:]
    net = Net(args.batch, seed=args.seed)
    steps_per_epoch = train_idx.numel() // args.batch
    total = steps_per_epoch * args.epochs
    xb = torch.empty((args.batch, 4, HW), dtype=torch.float32, device="cuda")
    yb = torch.empty((args.batch, 3, HW), dtype=torch.float32, device="cuda")
    out = torch.empty((args.batch, 3, HW), dtype=torch.float32, device="cuda")

    def validate():
        tot, cnt = 0.0, 0
        for s in range(0, n_val - args.batch + 1, args.batch):
            idx = val_idx[s:s + args.batch]
            xb.copy_(inputs[idx])
            net.forward(args.batch, xb.data_ptr(), out.data_ptr())
            tot += masked_mse(torch, out, labels[idx], xb)
            cnt += 1
        return tot / max(cnt, 1)

    zero_val = masked_mse(torch, torch.zeros_like(labels[val_idx]), labels[val_idx], inputs[val_idx])
    record = dict(pairs=n, val_pairs=n_val, epochs=args.epochs, batch=args.batch, lr=args.lr,
                  val_mse_zero_prediction=zero_val, epochs_log=[])
    log(f"validation MSE of the zero prediction: {zero_val:.5f}")
    step = 0
    t_train = time.time()
    for ep in range(args.epochs):
        order = train_idx[torch.randperm(train_idx.numel(), generator=g, device="cuda")]
        losses = []
        for s in range(steps_per_epoch):
            idx = order[s * args.batch:(s + 1) * args.batch]
            xb.copy_(inputs[idx])
            yb.copy_(labels[idx])
            lr = args.lr_min + 0.5 * (args.lr - args.lr_min) * (1 + math.cos(math.pi * step / max(total, 1)))
            losses.append(net.train_step(args.batch, xb.data_ptr(), yb.data_ptr(), lr))
            step += 1
        v = validate()
        record["epochs_log"].append(dict(epoch=ep + 1, train_mse=float(np.mean(losses)), val_mse=v))
        log(f"epoch {ep + 1}: train {np.mean(losses):.5f}  val {v:.5f}  ({time.time() - t_train:.1f} s)")
    record["train_seconds"] = time.time() - t_train
    record["total_seconds"] = time.time() - t_start
    params = net.get_params()
    np.savez(args.out, params=params, record=json.dumps(record))
    log(f"wrote {args.out} ({params.size} parameters)")
    net.close()
    return record


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-min", type=float, default=5e-5)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default="warmstart.npz")
    train(ap.parse_args())


if __name__ == "__main__":
    main()
