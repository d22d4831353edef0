"""Properties of the C-grid oracle and of the host-side C-grid initial state
(CPU only).  The oracle's operators are pinned to the reference's printed
values in test_oracle_golden.py; these tests add the SBP properties the
reference's C-grid scheme is built for."""
import numpy as np
import pytest

import oracle
from cubedsphere_sbp_swm_gb300 import initial


@pytest.mark.parametrize("mesh", ["p", "u", "v", "q"])
def test_host_geometry_matches_oracle_meshes(mesh):
    N = 20
    od = oracle.OracleCDomain(N, 42)
    g = initial.ecs_geometry(N, "ah" if mesh == "q" else mesh)
    x, y, z = od.points(mesh)
    assert np.array_equal(g["r"], np.stack([x, y, z], -1))
    assert np.array_equal(g["J"], od.metric(mesh)["J"])
    b = od.bases(mesh)
    assert np.abs(g["a1"] - b["a1"]).max() < 1e-15 and np.abs(g["a2"] - b["a2"]).max() < 1e-15


@pytest.mark.parametrize("order", [42, 21])
def test_sbp_mass_conservation(order):
    """SBP-SAT divergence with the SBP_C quadrature: the global integral of
    the h tendency vanishes to round-off for any state."""
    N = 24
    od = oracle.OracleCDomain(N, order)
    h, u, v, _ = initial.balanced_zonal_c(N, 4, 10)
    rng = np.random.default_rng(1)
    u = u + rng.standard_normal(u.shape)
    v = v + rng.standard_normal(v.shape)
    th, _, _ = od.apply(h, u, v)
    assert abs(od.mass(th)) / od.mass(np.abs(th)) < 1e-13


@pytest.mark.parametrize("order", [42, 21])
def test_balanced_flow_stays_balanced(order):
    """The balanced zonal flow is a steady solution: after a day of RK4 steps
    the height changes by far less than its own variation, and the mass is
    kept to round-off.  dt = 600 s at N = 24 (Courant number about 0.4 for
    the gravity waves); the 4/2 scheme turns unstable near 1000 s there."""
    N = 24
    od = oracle.OracleCDomain(N, order)
    h, u, v, _ = initial.balanced_zonal_c(N, 2, 0, pert_rms=0.0)
    m0 = od.mass(h)
    h1, u1, v1 = od.rk4(h, u, v, 600.0, 144)
    assert np.all(np.isfinite(h1)) and np.all(np.isfinite(u1))
    assert np.abs(h1 - h).max() < 0.02 * (h.max() - h.min())
    assert abs(od.mass(h1) - m0) / m0 < 1e-13


def test_sbp42_more_accurate_than_sbp21():
    """The 4/2 operators converge faster than the 2/1 ones on the same
    smooth field (test_diffops_conv.f90's premise): compare the cross-polar
    divergence errors at N=32."""
    e42 = oracle.golden_c("div", 32, 42)
    e21 = oracle.golden_c("div", 32, 21)
    assert e42[3] < e21[3]
    g42, g21 = oracle.golden_c("grad", 32, 42), oracle.golden_c("grad", 32, 21)
    assert g42[1] < 0.1 * g21[1]
