"""Solve one synthetic batch and exit: the fixed workload profilers attach to.

    python -m pdflow.solve_once --rows 480 --batch 64 [--form 2] [--solves 2]

Renders a few seeded scenes (repeated to fill the batch), pushes both frames
and runs `--solves` batched solves without CUDA graphs, so a kernel profiler
sees every launch of every level.  Prints the flow checksum of pair 0.
"""
from __future__ import annotations

import argparse

import numpy as np

from . import BatchSolver, Net, load_weights, scenes


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--rows", type=int, default=480, choices=(60, 120, 240, 480))
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--form", type=int, default=10, choices=tuple(range(11)))
    ap.add_argument("--learned", type=float, default=0.0,
                    help="iteration scale of a learned warm-started solve (0: plain solve)")
    ap.add_argument("--solves", type=int, default=2)
    ap.add_argument("--copy-mode", type=int, default=-1, choices=(-1, 0, 1, 2, 3),
                    help="tile region copies of the chosen paired form (bit 0 bulk load, bit 1 bulk store; -1: default)")
    ap.add_argument("--distinct", type=int, default=4)
    a = ap.parse_args()
    if a.copy_mode >= 0 and a.form >= 3:
        from . import _lib
        _lib.check(_lib.load().pdflow_set_tile_copy_mode(a.form - 3, a.copy_mode), "pdflow_set_tile_copy_mode")
    vga = a.rows == 480
    w, h = (640, 480) if vga else (320, 240)
    pairs = [scenes.make_pair(1000 + k, vga=vga) for k in range(a.distinct)]
    stack = lambda j: np.stack([pairs[k % a.distinct][j] for k in range(a.batch)])
    b = BatchSolver(a.rows, w, h, a.batch, use_graph=False, iteration_form=a.form)
    b.push_raw(stack(0), stack(1))
    b.push_raw(stack(2), stack(3))
    net = None
    if a.learned > 0:
        net = Net(a.batch)
        net.set_params(load_weights())
    for _ in range(a.solves):
        if net is not None:
            b.solve_learned(a.batch, net, a.learned, 0.01)
        else:
            b.solve(a.batch)
    dx, dy, dz = b.read_flow(1)
    b.close()
    if net is not None:
        net.close()
    print(f"rows={a.rows} batch={a.batch} form={a.form}: sum|dx|+|dy|+|dz| of pair 0 = "
          f"{float(np.abs(dx).sum() + np.abs(dy).sum() + np.abs(dz).sum()):.6f}")


if __name__ == "__main__":
    main()
