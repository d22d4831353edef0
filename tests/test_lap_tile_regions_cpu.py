"""The FP32 narrow Laplacian's tile regions, restated on the CPU (no GPU).

lap_tile_kernel (csrc/swm_diffusion.cu) stages a region of each 32 x 8 node
tile in shared arrays sized at compile time (LapTile: RX columns, RY rows)
and finishes every node of the tile from them.  This restates its tile
placement (the last tile of a line moved back to end on the panel edge),
lap_region's arithmetic and the LapTile sizes, and checks for every panel
size the library accepts (N = 16 .. 2100, n = N + 1 nodes) and the three
narrow orders that
- every region fits its shared array, and
- every stencil a tile node reads lies in the region: the narrow D2 row
  (closure rows read the first / last cols nodes, the interior +-hw) and the
  SBP first derivative of the same order at the node (closure rows read the
  first / last NW nodes, the interior +-H), which is also the stencil of the
  mixed terms along the other direction.
The table shapes are read from the generated header."""
import functools
import os
import re

import pytest

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "cubedsphere_sbp_swm_gb300", "csrc", "swm_narrow_tables.h")
LTX, LTY = 32, 8
# SBP first-derivative shapes (closure rows NE, their width NW, interior
# half width H) of the orders 2/1, 4/2 and 6/3
SBP = {21: (1, 2, 1), 42: (4, 6, 2), 63: (6, 9, 3)}


@functools.lru_cache(maxsize=None)
def _shape(order):
    txt = open(HDR).read()
    m = re.search(r"constexpr NarrowD2 kNarrow%d = \{\s*(\d+), (\d+), (\d+), (\d+), (\d+)," % order, txt)
    assert m, order
    o, rows, cols, nb, hw = map(int, m.groups())
    assert o == order
    return rows, cols, hw


@functools.lru_cache(maxsize=None)
def _sizes(order):
    rows, cols, hw = _shape(order)
    H1 = SBP[order][2]
    R = max(hw, H1)
    EXT = R + max(R, rows - 1)
    return R, LTX + EXT, LTY + max(EXT, 2 * rows - 2)


def _region(order, a0, ln, n):
    rows, cols, _ = _shape(order)
    R = _sizes(order)[0]
    lo, hi = max(0, a0 - R), min(n, a0 + ln + R)
    if a0 < rows:
        lo, hi = 0, max(hi, min(n, cols))
    if a0 + ln > n - rows:
        hi, lo = n, min(lo, max(0, n - cols))
    return lo, hi


def _needs(order, k, n):
    """[first, last] node a tile node k reads along the line."""
    rows, cols, hw = _shape(order)
    NE, NW, H = SBP[order]
    if k < rows:
        a, b = 0, cols - 1
    elif k >= n - rows:
        a, b = n - cols, n - 1
    else:
        a, b = k - hw, k + hw
    if k < NE:
        c, d = 0, NW - 1
    elif k >= n - NE:
        c, d = n - NW, n - 1
    else:
        c, d = k - H, k + H
    return min(a, c), max(b, d)


@pytest.mark.parametrize("order", [21, 42, 63])
def test_regions_fit_and_hold_every_stencil(order):
    rows, cols, hw = _shape(order)
    _, RX, RY = _sizes(order)
    assert rows >= SBP[order][0]   # tiles without closure nodes take the interior D1
    for N in range(16, 2101):
        n = N + 1
        if n < 2 * rows:
            continue
        for L, cap in ((LTX, RX), (LTY, RY)):
            ln = min(L, n)
            for b in range((n + L - 1) // L):
                a0 = min(b * L, n - ln)
                lo, hi = _region(order, a0, ln, n)
                assert 0 <= lo and hi <= n and hi - lo <= cap, (order, N, L, a0, lo, hi, cap)
                # the tile's end nodes and its closure nodes (the interior
                # nodes between read inside the end nodes' span)
                ks = {a0, a0 + 1, a0 + ln - 2, a0 + ln - 1}
                ks.update(k for k in range(a0, min(a0 + ln, rows)))
                ks.update(k for k in range(max(a0, n - rows), a0 + ln))
                for k in ks:
                    if a0 <= k < a0 + ln:
                        a, z = _needs(order, k, n)
                        assert lo <= a and z < hi, (order, N, L, a0, k, a, z, lo, hi)
