"""The stage kernel's work split (host logic, no device work): every node of
every panel is owned by exactly one unit, each unit reads a range that holds
its own nodes and the stencils they need and fits the consumer width, the
automatic split fills at most one wave, and the cost model gives strips on
a panel edge and the closure rows smaller units."""
import ctypes

import numpy as np
import pytest

from cubedsphere_sbp_swm_gb300 import _abi


def _split(N, order, cols, target, seg_rows=0):
    L = _abi.load()
    cap = 20000
    out = (ctypes.c_int * (9 * cap))()
    n_units = ctypes.c_int()
    rc = L.swm_work_split(N, order, cols, target, seg_rows, out, cap, ctypes.byref(n_units))
    assert rc == 0, rc
    return np.frombuffer(out, dtype=np.int32)[: 9 * n_units.value].reshape(-1, 9)


# closure rows (ne) and interior half width (H) of the SBP first derivative
SHAPES = {21: (1, 1), 42: (4, 2), 43: (4, 2), 63: (6, 3)}


@pytest.mark.parametrize("N,order,cols,target,seg", [
    (384, 42, 128, 456, 0), (384, 42, 64, 760, 0), (1024, 63, 96, 456, 0), (1024, 63, 128, 304, 0),
    (48, 42, 64, 760, 0), (96, 43, 96, 456, 0), (40, 63, 128, 456, 0), (16, 21, 64, 456, 0),
    (384, 42, 128, 456, 24), (1024, 63, 96, 456, 64), (192, 42, 160, 1, 96), (48, 42, 96, 1, 0),
])
def test_units_partition_every_panel(N, order, cols, target, seg):
    n = N + 1
    U = _split(N, order, cols, target, seg)
    own = np.zeros((6, n, n), dtype=np.int32)
    for p, i0, i1, j0, j1, cl0, cl1, rl0, rl1 in U:
        assert 0 <= p < 6 and 0 <= i0 < i1 <= n and 0 <= j0 < j1 <= n
        own[p, j0:j1, i0:i1] += 1
        # the read range holds the owned nodes, stays in the panel and fits
        # the consumer threads
        assert 0 <= cl0 <= i0 and i1 <= cl1 <= n and cl1 - cl0 <= cols
        assert 0 <= rl0 <= j0 and j1 <= rl1 <= n
    assert (own == 1).all(), "every node owned by exactly one unit"
    if seg == 0:
        nstrip = len(np.unique(U[:, 1]))
        assert len(U) <= max(target, 6 * nstrip)


def test_cost_model_gives_edge_strips_and_closure_rows_fewer_rows():
    N, n = 384, 385
    U = _split(N, 42, 128, 456)
    assert len(U) <= 456
    edge = (U[:, 1] == 0) | (U[:, 2] == n)
    rows = U[:, 4] - U[:, 3]
    assert rows[edge].mean() < rows[~edge].mean()
    inner = ~edge & (U[:, 0] == 0)
    order = np.argsort(U[inner, 3])
    r = rows[inner][order]
    assert r[0] < np.median(r) and r[-1] < np.median(r)   # closure rows at both ends


def test_fixed_rows_per_unit():
    N, n = 384, 385
    U = _split(N, 42, 128, 1, seg_rows=32)
    edge = (U[:, 1] == 0) | (U[:, 2] == n)
    per_strip = {}
    for u, e in zip(U, edge):
        if u[0] == 0:
            per_strip.setdefault((u[1], bool(e)), 0)
            per_strip[(u[1], bool(e))] += 1
    inner_counts = [c for (i0, e), c in per_strip.items() if not e]
    edge_counts = [c for (i0, e), c in per_strip.items() if e]
    assert all(c == 13 for c in inner_counts)          # ceil(385 / 32) units
    assert all(c == 17 for c in edge_counts)           # 1.3 x as many on the panel edges


def test_bad_arguments():
    L = _abi.load()
    out = (ctypes.c_int * 9)()
    nu = ctypes.c_int()
    assert L.swm_work_split(384, 42, 128, 456, 0, out, 1, ctypes.byref(nu)) == _abi.SWM_E_INVALID
    assert L.swm_work_split(384, 44, 128, 456, 0, out, 1, ctypes.byref(nu)) == _abi.SWM_E_UNSUPPORTED
    assert L.swm_work_split(4, 42, 128, 456, 0, out, 1, ctypes.byref(nu)) == _abi.SWM_E_INVALID
