"""Generates the golden vectors of tests/golden/ by running the reference's own
CUDA path (oracle/_ref/pdflow_ref.cubin through oracle/ref/refharness.c) on
seeded synthetic RGB-D pairs.  Needs a GPU and the reference device code:

    make -C oracle/ref                      # where the reference sources exist
    python tests/golden/make_golden.py --out golden_new   # on a GPU; then copy the .npz files here

Each fixture stores the uint8/uint16 row-major input images (so the tests do
not depend on the scene generator being bit-identical across machines) and the
reference's outputs, float32:

  qvga_s0.npz  QVGA pair (seed 0, 3 objects): flow for rows=240 and rows=60,
               plus per-level intermediates of the rows=60 solve
  vga_s2.npz   VGA pair (seed 2, 6 objects): flow for rows=480 and rows=240

It also solves each case twice and records whether the reference repeats
itself bit for bit (`repeatable_*`).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "pd-flow_gb300"))

from oracle import refharness  # noqa: E402
from pdflow import scenes  # noqa: E402

# intermediates kept for the small case (levels 0..2 of rows=60)
DUMP_KEEP = ("dct", "dcu", "dcv", "ddt", "ddu", "ddv", "mu", "ri", "rj", "ri_2", "rj_2", "du_prev", "dv_prev",
             "sigma_pd", "sigma_puvx", "sigma_puvy", "sigma_pwx", "sigma_pwy", "tau_u", "tau_v", "tau_w",
             "init_dw", "init_pd", "init_puu", "init_puv", "init_pvu", "init_pvv", "init_pwu", "init_pwv",
             "du_new", "dv_new", "dw_new", "du_acc", "dv_acc", "dw_acc", "pd", "puu", "puv", "pvu", "pvv", "pwu",
             "pwv", "sat_du", "sat_dv", "sat_dw", "du_l", "dv_l", "dw_l")


def solve_case(rows, w, h, I1, Z1, I2, Z2, dump=False):
    s = refharness.RefSolver(rows, w, h)
    try:
        out = s.solve_pair(I1, Z1, I2, Z2, dump=dump)
        again = s.solve_pair(I1, Z1, I2, Z2)
    finally:
        s.close()
    rep = all(np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in zip(out[:3], again[:3]))
    return out, rep


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default="golden_new")
    args = ap.parse_args()
    os.makedirs(args.out, exist_ok=True)

    # QVGA pair
    i1, z1, i2, z2 = scenes.make_pair(0, vga=False, n_objects=3)
    I1, Z1 = scenes.decode(i1, z1)
    I2, Z2 = scenes.decode(i2, z2)
    rec = dict(i1=i1, z1=z1, i2=i2, z2=z2)
    (dx, dy, dz), rep = solve_case(240, 320, 240, I1, Z1, I2, Z2)
    rec.update(r240_dx=dx, r240_dy=dy, r240_dz=dz, repeatable_r240=np.array(rep))
    (dx, dy, dz, store), rep = solve_case(60, 320, 240, I1, Z1, I2, Z2, dump=True)
    rec.update(r60_dx=dx, r60_dy=dy, r60_dz=dz, repeatable_r60=np.array(rep))
    for (name, level), arr in store.items():
        base = name[4:] if name.startswith("old_") else name
        if base.startswith("push_"):
            # pyramid levels 2.. of both frames (80x60 and coarser)
            if level >= 2:
                rec[f"r60_{name}_L{level}"] = arr
        elif name in DUMP_KEEP:
            rec[f"r60_{name}_L{level}"] = arr
    np.savez_compressed(os.path.join(args.out, "qvga_s0.npz"), **rec)
    print("qvga_s0 repeatable:", bool(rec["repeatable_r240"]), bool(rec["repeatable_r60"]))

    # VGA pair
    i1, z1, i2, z2 = scenes.make_pair(2, vga=True, n_objects=6)
    I1, Z1 = scenes.decode(i1, z1)
    I2, Z2 = scenes.decode(i2, z2)
    rec = dict(i1=i1, z1=z1, i2=i2, z2=z2)
    for rows in (480, 240):
        (dx, dy, dz), rep = solve_case(rows, 640, 480, I1, Z1, I2, Z2)
        rec.update({f"r{rows}_dx": dx, f"r{rows}_dy": dy, f"r{rows}_dz": dz, f"repeatable_r{rows}": np.array(rep)})
    np.savez_compressed(os.path.join(args.out, "vga_s2.npz"), **rec)
    print("vga_s2 repeatable:", bool(rec["repeatable_r480"]), bool(rec["repeatable_r240"]))

    # timing of the reference CUDA path (pairs/s), for the record
    for vga, rows in ((False, 240), (True, 480)):
        i1, z1, i2, z2 = scenes.make_pair(5, vga=vga)
        I1, Z1 = scenes.decode(i1, z1)
        I2, Z2 = scenes.decode(i2, z2)
        w, h = (640, 480) if vga else (320, 240)
        s = refharness.RefSolver(rows, w, h)
        s.time_pairs(I1, Z1, I2, Z2, 2)
        ms = s.time_pairs(I1, Z1, I2, Z2, 10)
        s.close()
        print(f"reference CUDA path rows={rows} {w}x{h}: {ms:.3f} ms/pair, {1000.0 / ms:.2f} pairs/s")


if __name__ == "__main__":
    main()
