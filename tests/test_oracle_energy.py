"""The oracle's energy functional and seeded solve (CPU only).

The energy is what the learned warm start's fallback rule compares; the seeded
solve is the CPU restatement of the warm-started coarse-to-fine path."""
import numpy as np
import pytest

from oracle import oracle
from pdflow import scenes


@pytest.fixture(scope="module")
def qvga60():
    i1, z1, i2, z2 = scenes.make_pair(11, vga=False, n_objects=3)
    I1, Z1 = scenes.decode(i1, z1)
    I2, Z2 = scenes.decode(i2, z2)
    dx, dy, dz, st = oracle.solve(60, 320, 240, I1, Z1, I2, Z2, precision="f64", dump=True)
    return (I1, Z1, I2, Z2), st


def level(st, li, frame):
    tag = "pyr_new_" if frame else "pyr_old_"
    return tuple(st[(tag + k, li)] for k in ("colour", "depth", "xx", "yy"))


def test_energy_of_the_solution_is_below_the_energy_of_zero_flow(qvga60):
    _, st = qvga60
    R, C, i, li = 60, 80, 2, 2          # finest solved level of rows=60 is image level 2 (80x60)
    old, new = level(st, li, 0), level(st, li, 1)
    du, dv, dw = st[("du_l", i)], st[("dv_l", i)], st[("dw_l", i)]
    e_sol = oracle.energy(R, C, old, new, du, dv, dw)
    z = np.zeros(R * C)
    e_zero = oracle.energy(R, C, old, new, z, z, z)
    assert 0 < e_sol < e_zero
    e32 = oracle.energy(R, C, old, new, du, dv, dw, precision="f32")
    assert abs(e32 - e_sol) <= 1e-4 * e_sol


def test_seeded_solve_from_the_plain_level_solution_stays_close(qvga60):
    (I1, Z1, I2, Z2), st = qvga60
    # rows=120: levels 15x20, 30x40, 60x80, 120x160; seed level 2 from the plain
    # rows=120 solve's own level-2 output
    dx, dy, dz, st120 = oracle.solve(120, 320, 240, I1, Z1, I2, Z2, precision="f64", dump=True)
    seed = np.concatenate([st120[(k, 2)] for k in ("du_l", "dv_l", "dw_l")]).astype(np.float32)
    sx, sy, sz = oracle.solve_seeded(120, 320, 240, I1, Z1, I2, Z2, 2, seed, 1.0)
    valid = st120[("pyr_old_depth", 1)] > 0
    epe = np.sqrt((sx - dx) ** 2 + (sy - dy) ** 2 + (sz - dz) ** 2)[valid]
    assert epe.mean() < 2e-3          # metres: same level-3 problem, different duals / start


def test_seeded_solve_rejects_level_zero():
    i1, z1, i2, z2 = scenes.make_pair(3)
    I1, Z1 = scenes.decode(i1, z1)
    I2, Z2 = scenes.decode(i2, z2)
    with pytest.raises(ValueError):
        oracle.solve_seeded(60, 320, 240, I1, Z1, I2, Z2, 0, np.zeros(3 * 300, np.float32))
