"""Pin the FP64 oracle against the reference's own known-answer tests.

The reference prints operator error norms at N=32, nz=3 on the unit sphere
(src/test/test_diff_ops/test_diffops_all.f90) and diffs them against
reference_results.txt; tests/golden/diffops_ah_n32.json holds the Ah-grid
lines of that file.  The oracle must reproduce every SBP operator value to
the 7 printed significant digits.  The colocated co2contra, contra2co,
Coriolis and kinetic-energy values are pure roundoff (3e-16 .. 2e-15) and
depend on the compiler's operation order, so they are checked as
roundoff-level only (within 1e-15 of the printed value).
"""
import json
import os

import numpy as np
import pytest

import oracle

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "diffops_ah_n32.json")))


def _fmt7(x):
    return "%.6E" % x  # the reference prints E15.7 (0.ddddddd): 7 significant digits


@pytest.mark.parametrize("entry", [g for g in GOLDEN if g["kind"] in ("div", "grad", "curl")],
                         ids=lambda g: g["name"])
def test_sbp_operator_golden_7_digits(entry):
    got = oracle.golden(entry["kind"], entry["N"], entry["sbp_order"])
    want = entry["values"]
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert _fmt7(g) == _fmt7(w), f"{entry['name']}: {g!r} vs {w!r} ({entry['source']})"


@pytest.mark.parametrize("entry", [g for g in GOLDEN if g["kind"] in ("co2contra", "contra2co", "coriolis", "ke")],
                         ids=lambda g: g["name"])
def test_colocated_transform_roundoff(entry):
    got = oracle.golden(entry["kind"], entry["N"])
    for g, w in zip(got, entry["values"]):
        assert g < 1e-14 and w < 1e-14
        assert abs(g - w) < 1e-15


@pytest.mark.parametrize("order,max_degree", [(21, 1), (42, 3), (63, 5)])
def test_sbp_quadrature_exactness(order, max_degree):
    # test_quadrature_mod.f90:18-80 (tolerance 1e-12; Ah21 to degree 1, Ah42
    # to degree 3).  Ah63 is not tested by the reference; degree 5 is the
    # exactness its 6/3 diagonal norm carries.
    assert oracle.quadrature_error(20, order, max_degree) < 1e-12


def test_rk4_iomega_amplification():
    # test_time_steping/test_ts_mod.f90:37-73: sum |f - f_true| < 1e-12
    assert oracle.rk4_iomega_error() < 1e-12


def test_halo_ring_scalar_copies_duplicated_node():
    # The exchanged 1-wide ring holds the neighbour's copy of the physically
    # same edge node (exchange_factory_mod.f90:157-299): syncing a continuous
    # field (here the Cartesian coordinates) must leave it unchanged.
    d = oracle.OracleDomain(16, 42, radius=1.0, omega=1.0)
    g = d.geometry()
    for key in ("rx", "ry", "rz"):
        synced = d.sync_scalar(g[key])
        assert np.max(np.abs(synced - g[key])) < 1e-15


def test_vector_sync_keeps_tangential_covariant_component():
    # The covariant component along a cube edge is the same on both panels,
    # so the exchange (with its swap/negation) followed by the plain average
    # keeps it; only the normal component gets the metric-weighted average.
    d = oracle.OracleDomain(16, 42, radius=1.0, omega=1.0)
    b = d.bases()
    w = np.array([0.3, -0.7, 0.2])
    g = d.geometry()
    r = np.stack([g["rx"], g["ry"], g["rz"]], -1)
    vec = np.cross(w, r)                       # smooth tangent field
    u = np.einsum("pjic,pjic->pji", vec, b["a1"]).copy()
    v = np.einsum("pjic,pjic->pji", vec, b["a2"]).copy()
    gx, gy = d.sync_vector_cov(u, v)
    n = d.n
    # left/right edges: the tangential covariant component is v (beta)
    assert np.max(np.abs(gy[:, 1:n - 1, 0] - v[:, 1:n - 1, 0])) < 1e-14
    assert np.max(np.abs(gy[:, 1:n - 1, n - 1] - v[:, 1:n - 1, n - 1])) < 1e-14
    # bottom/top edges: the tangential covariant component is u (alpha)
    assert np.max(np.abs(gx[:, 0, 1:n - 1] - u[:, 0, 1:n - 1])) < 1e-14
    assert np.max(np.abs(gx[:, n - 1, 1:n - 1] - u[:, n - 1, 1:n - 1])) < 1e-14
    # and the whole field, a smooth exact vector, is reproduced closely
    assert np.max(np.abs(gx - u)) < 1e-12 and np.max(np.abs(gy - v)) < 1e-12


def test_discrete_mass_conservation():
    # SBP divergence + SBP quadrature: the global integral of dh/dt vanishes
    # to roundoff for any smooth state (consequence of summation by parts).
    d = oracle.OracleDomain(24, 42)
    g = d.geometry()
    b = d.bases()
    r = np.stack([g["rx"], g["ry"], g["rz"]], -1)
    vel = 30.0 * np.cross([0.2, 0.1, 1.0], r)
    u = np.einsum("pjic,pjic->pji", vel, b["a1"]).copy()
    v = np.einsum("pjic,pjic->pji", vel, b["a2"]).copy()
    h = 5000.0 + 100.0 * g["rz"] * g["rx"]
    th, tu, tv = d.apply(h, u, v)
    scale = d.mass(np.abs(th)) + 1e-300
    assert abs(d.mass(th)) / scale < 1e-12


GOLDEN_C = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "diffops_c_n32.json")))


@pytest.mark.parametrize("entry", GOLDEN_C, ids=lambda g: g["name"])
def test_c_grid_operator_golden_7_digits(entry):
    """The C-grid SBP operators of the &shallow_water_model_c family
    (namelist_swm:80-102) against the reference's printed values, to the 7
    significant digits printed (reference_results.txt, test_diffops_all.f90
    at N=32, nz=3)."""
    got = oracle.golden_c(entry["kind"], entry["N"], entry["sbp_order"])
    want = entry["values"]
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert _fmt7(g) == _fmt7(w), f"{entry['name']}: {g!r} vs {w!r} ({entry['source']})"


REGRID = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "regrid_ah_n32.json")))


@pytest.mark.parametrize("case", REGRID, ids=lambda c: f"{c['kind']}-{c['components']}-{c['interp']}")
def test_latlon_regrid_matches_reference(case):
    """The reference's lat-lon regrid known-answer values (full precision,
    test_regrid_mod.f90 at N=32, Ah grid): maximum interpolation errors of
    the xyz scalar field and of the solid rotation field."""
    kind = case["components"] or "scalar"
    got = oracle.golden_regrid(kind, case["interp"])
    ref = np.array(case["values"])
    assert np.allclose(got, ref, rtol=1e-9, atol=0.0), (got, ref)
