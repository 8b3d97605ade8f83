"""CPU model of the strip walk of the streamed tiles (iteration form 10,
`pd-flow_gb300/csrc/pdflow_ptiles.cu`: `segment`, `strip_at`, `next_tile`)
over the work units the launcher computes (`pdflow_strip_units`, the same
host function the launch uses).  For every size it checks that each column
of each 24-row band is stored exactly once, by a region in which that
column is exact after the launch's kk iterations.  Exactness follows a taint
model of the stencil along the columns: the dual step of a column reads the
primal state of the column to its right, the primal step reads the new dual
of the column to its left; a region's first column takes that left value
from the carry of the region before it, and its last columns read their own
storage (not exact) unless they are the image's last column."""
import ctypes
from functools import lru_cache

import numpy as np
import pytest

REGION = 32          # region columns (kSR)
BAND = 24            # exact rows of a band (the row halo is 4 >= kk)


def strip_units(lib, bands, cols, kk, ctas):
    whole = ctypes.c_uint()
    tn = (ctypes.c_uint * 3)()
    tp = (ctypes.c_uint * 3)()
    assert lib.pdflow_strip_units(bands, cols, kk, ctas, ctypes.byref(whole), tn, tp) == 0
    return whole.value, list(tn), list(tp)


def segment(units, cols, k):
    """Band and column range [c0, c1) of unit k (pdflow_ptiles.cu: segment)."""
    whole, tn, tp = units
    if k < whole:
        return k, 0, cols
    x, base = k - whole, whole
    for n, m in zip(tn, tp):
        if x < n * m:
            piece = x // n
            return base + x % n, cols * piece // m, cols * (piece + 1) // m
        x -= n * m
        base += n
    return None


@lru_cache(maxsize=None)
def region_exact(cols, kk, ru0, carry):
    """Exact columns of a region at ru0 after kk iterations, and the carry it
    hands on (the new dual of column REGION - 1 - kk per iteration).  `carry`
    is the tuple of the previous region's carry flags, or None."""
    us = [ru0 + c for c in range(REGION)]
    P = [u < cols for u in us]                       # loaded state: exact inside the image
    D = list(P)
    out = []
    for j in range(kk):
        nD = [u < cols and D[c] and P[c] and (u == cols - 1 or (c + 1 < REGION and P[c + 1]))
              for c, u in enumerate(us)]
        nP = []
        for c, u in enumerate(us):
            if u >= cols:
                nP.append(False)
                continue
            if u == 0:
                left = True
            elif c == 0:
                left = carry is not None and carry[j]
            else:
                left = nD[c - 1]
            nP.append(P[c] and nD[c] and left)
        D, P = nD, nP
        out.append(D[REGION - 1 - kk])
    return tuple(P[c] and D[c] for c in range(REGION)), tuple(out)


@lru_cache(maxsize=None)
def walk(cols, kk, c0, c1):
    """Columns stored by the regions of a unit [c0, c1) (strip_at/next_tile),
    after checking that each stored column is exact; returns (stored columns,
    regions walked)."""
    col, carry, carry_vals, stored, regions = c0, False, None, [], 0
    while True:
        ru0 = col if carry else max(col - kk, 0)
        exact = cols if ru0 + REGION >= cols else ru0 + REGION - kk
        iu1 = min(exact, c1)
        assert iu1 > col, (cols, kk, c0, c1, col)
        ex, out = region_exact(cols, kk, ru0, carry_vals if carry else None)
        for u in range(col, iu1):
            assert ex[u - ru0], (cols, kk, c0, c1, ru0, u)
        stored.append((col, iu1))
        regions += 1
        if iu1 >= c1:
            return tuple(stored), regions
        assert iu1 == exact                       # the next region continues with the carry
        assert exact - 1 - ru0 == REGION - 1 - kk  # of the column that wrote it
        col, carry, carry_vals = iu1, True, out


def check(lib, rows, cols, pairs, kk, ctas):
    bands = pairs * ((rows + BAND - 1) // BAND)
    units = strip_units(lib, bands, cols, kk, ctas)
    whole, tn, tp = units
    assert whole + sum(tn) == bands
    stored = np.zeros((bands, cols), np.int32)
    k = 0
    while True:
        sg = segment(units, cols, k)
        if sg is None:
            break
        band, c0, c1 = sg
        assert c1 > c0
        for a, b in walk(cols, kk, c0, c1)[0]:
            stored[band, a:b] += 1
        k += 1
    assert k == whole + sum(n * m for n, m in zip(tn, tp))
    assert (stored == 1).all(), (rows, cols, pairs, kk, ctas)


@pytest.mark.parametrize("rows,cols", [(60, 80), (120, 160), (240, 320), (480, 640), (4, 20), (32, 28), (64, 33),
                                       (8, 24), (480, 700)])
def test_every_band_column_stored_once_and_exact(built_lib, rows, cols):
    for pairs in (1, 3, 17, 64):
        for kk in (1, 2, 3, 4):
            for ctas in (1, 2, 7, 152):
                check(built_lib, rows, cols, pairs, kk, ctas)


def test_unit_tiers_of_the_batched_vga_levels(built_lib):
    """64 VGA pairs on 152 SMs at 4 iterations per launch: long bands (480x640,
    23 regions) end with 19 bands in 2 pieces, 19 in 4 and 38 in 8; the
    240x320 bands (12 regions) with 19 in each; fewer bands than CTAs are
    all cut into as many pieces as the CTAs allow."""
    assert strip_units(built_lib, 64 * 20, 640, 4, 152) == (1280 - 76, [19, 19, 38], [2, 4, 8])
    assert strip_units(built_lib, 64 * 10, 320, 4, 152) == (640 - 57, [19, 19, 19], [2, 4, 8])
    assert strip_units(built_lib, 20, 640, 4, 152) == (0, [20, 0, 0], [7, 4, 8])
    assert built_lib.pdflow_strip_units(0, 640, 4, 152, ctypes.byref(ctypes.c_uint()), (ctypes.c_uint * 3)(),
                                        (ctypes.c_uint * 3)()) != 0
