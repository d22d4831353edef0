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


# ---------------------------------------------------------------- hyperdiffusion
# operator_swm_diff_t with the &shallow_water_model_c names: hordiff_c_biharm_*
# for (u, v) and hordiff_scalar_C for h, always with the 2/1 operators
# (hordiff_factory_mod.f90:53-139, 196-247).

def test_hyperdiffusion_uses_the_2_1_operators_at_any_order():
    """The factory builds the C-grid hyperdiffusion from the sbp21 operators
    whatever the model's order, so a 4/2 domain gives the same tendency as a
    2/1 domain bit for bit."""
    N = 20
    d21, d42 = oracle.OracleCDomain(N, 21), oracle.OracleCDomain(N, 42)
    h, u, v, _ = initial.balanced_zonal_c(N, 5, 10)
    for name in ("hordiff_c_biharm_div", "hordiff_c_biharm_curl", "hordiff_c_biharm_curl_div"):
        a = d21.hordiff(h, u, v, name)
        b = d42.hordiff(h, u, v, name)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_hyperdiffusion_matches_the_biharmonic_away_from_panel_edges():
    """h = z and the solid rotation are l = 1 fields (Laplacian eigenvalue
    -2/a^2), so the exact tendency is -c^4 (2/a^2)^2 f = -4 coeff^4 hx^4 f.
    The 2/1 gradient's edge closure leaves the Laplacian O(1) wrong on the
    edge rows (the reference's own gradient_c_sbp21 error is 7% at N=32), so
    the comparison starts four rows in, where the error converges."""
    errs = []
    for N in (24, 48):
        d = oracle.OracleCDomain(N, 21)
        hx = np.pi / 2 / N
        lam = -4 * 0.03 ** 4 * hx ** 4
        z = d.scalar_test_field("xyz", 2, "p")
        u, v = d.vector_test_field("solid_rotation", 0)
        th, tu, tv = d.hordiff(z, u, v, "hordiff_c_biharm_curl_div", 0.03, 0.03)
        eh = (th - lam * z).reshape(6, N, N)[:, 4:-4, 4:-4]
        eu = (tu - lam * u).reshape(6, N, N + 1)[:, 4:-4, 4:-4]
        ev = (tv - lam * v).reshape(6, N + 1, N)[:, 4:-4, 4:-4]
        errs.append((np.abs(eh).max() / np.abs(lam * z).max(),
                     max(np.abs(eu).max(), np.abs(ev).max()) / np.abs(lam * u).max()))
    assert errs[0][0] < 0.02 and errs[0][1] < 0.05
    assert errs[1][0] < 0.5 * errs[0][0] and errs[1][1] < 0.5 * errs[0][1]


def test_hyperdiffusion_conserves_mass_and_dissipates():
    """The h part is a divergence, so its SBP_C21 integral vanishes; it is
    negative semi-definite (<h, D h> < 0), and every vector part lowers the
    kinetic energy of a rough flow in one explicit Euler step."""
    N = 24
    d = oracle.OracleCDomain(N, 21)
    rng = np.random.default_rng(3)
    h0, u0, v0, _ = initial.balanced_zonal_c(N, 4, 10)
    u0 = u0 + rng.standard_normal(u0.shape)
    v0 = v0 + rng.standard_normal(v0.shape)
    h = rng.standard_normal(h0.shape)
    th, _, _ = d.hordiff(h, u0, v0)
    assert abs(d.mass(th)) / d.mass(np.abs(th)) < 1e-13
    assert d.mass(h * th) < -0.5 * d.mass(np.abs(h * th))

    def ke(u, v):
        ut, vt = d.co2contra(u, v)
        return d.mass(d.ke(u, v, ut, vt))

    k0 = ke(u0, v0)
    for name in ("hordiff_c_biharm_div", "hordiff_c_biharm_curl", "hordiff_c_biharm_curl_div"):
        _, tu, tv = d.hordiff(h0, u0, v0, name)
        assert ke(u0 + 900.0 * tu, v0 + 900.0 * tv) < (1 - 1e-5) * k0


@pytest.mark.parametrize("order", [21, 42])
def test_grad_perp_is_divergence_free(order):
    """The staggered differences commute, so the divergence of grad_perp of
    any corner field vanishes to round-off (the mimetic property the curl
    part of the hyperdiffusion relies on; a sign error in either component
    would leave 2 D_x D_y w)."""
    N = 24
    d = oracle.OracleCDomain(N, order)
    w = d.scalar_test_field("xyz", 2, "q") + 0.1 * d.scalar_test_field("cross_polar_zeta", 0, "q")
    gu, gv = d.grad_perp(w)
    scale = np.abs(gu).max() / (6.371e6 * np.pi / 2 / N)
    assert np.abs(d.div(gu, gv)).max() < 1e-13 * scale


@pytest.mark.parametrize("order", [21, 42])
def test_model_step_with_hyperdiffusion(order):
    """A day of the drivers' step (RK4, then the explicit Euler step of the
    hyperdiffusion with the namelist's coefficients 0.03) keeps the balanced
    flow balanced.  The mass is kept to round-off at 2/1; at 4/2 the 2/1
    divergence of the h diffusion is measured with the SBP_C42 quadrature,
    so it drifts at the 1e-8 level, as in the reference."""
    N = 24
    d = oracle.OracleCDomain(N, order)
    h, u, v, _ = initial.balanced_zonal_c(N, 2, 0, pert_rms=0.0)
    m0 = d.mass(h)
    h1, u1, v1 = d.model_step(h, u, v, 600.0, 144)
    assert np.all(np.isfinite(h1)) and np.all(np.isfinite(u1)) and np.all(np.isfinite(v1))
    assert np.abs(h1 - h).max() < 0.01 * (h.max() - h.min())
    assert abs(d.mass(h1) - m0) / m0 < (1e-13 if order == 21 else 1e-7)


# ------------------------------------------------------------------- ECS_O
# The interpolating ECS_O halo of the cell centres (equiang_cs/ecs_halo_mod.f90
# :95-475).  Its width-1 form is pinned by gradient_a2_ecs's known answer
# (test_oracle_golden.py); the reference's own halo test prints its errors
# without known answers, so the width-2 form is checked here against the
# exact field at the virtual points.

def _extended_points(N, hw):
    """Cartesian points of the extended panel grid lines, (6, W, W, 3)."""
    import math
    hx = 0.5 * math.pi / N
    a = -0.25 * math.pi + hx * (np.arange(1 - hw, N + hw + 1) - 0.5)
    ta, tb = np.tan(a)[None, :], np.tan(a)[:, None]
    sg = np.sqrt(1 + ta * ta + tb * tb)
    one = np.ones_like(sg)
    rp = np.stack([ta * one / sg, tb * one / sg, one / sg], -1)
    return (rp[None, ..., 0:1] * initial._EX[:, None, None, :] + rp[None, ..., 1:2] * initial._EY[:, None, None, :]
            - rp[None, ..., 2:3] * initial._EN[:, None, None, :])


@pytest.mark.parametrize("hw", [1, 2])
def test_ecs_o_halo_is_fourth_order(hw):
    """Edge rows, the points next to each cube corner and the points inside
    it all converge at fourth order to the exact field (errors fall by more
    than 12x per doubling of N); the interior is the field itself."""
    errs = []
    for N in (24, 48):
        od = oracle.OracleCDomain(N, 42, radius=1.0)
        r = _extended_points(N, hw)
        e = 0.0
        for lev in range(3):
            f = od.scalar_test_field("xyz", lev, "p")
            E = od.ecs_o_halo(f, hw)
            assert np.array_equal(E[:, hw:hw + N, hw:hw + N], f.reshape(6, N, N))
            e = max(e, float(np.abs(E - r[..., lev]).max()))
        errs.append(e)
    assert errs[0] < 3e-6 and errs[1] < errs[0] / 12.0, errs


def test_grad_a2_ecs_is_second_order():
    """gradient_a2_ecs converges at second order to the exact covariant
    gradient of x on the unit sphere."""
    errs = []
    for N in (24, 48):
        od = oracle.OracleCDomain(N, 42, radius=1.0)
        f = od.scalar_test_field("xyz", 0, "p")
        gx, gy = od.grad_a2_ecs(f)
        x, y, z = od.points("p")
        r = np.stack([x, y, z], -1)
        W = np.array([1.0, 0.0, 0.0]) - r[..., 0:1] * r
        b = od.bases("p")
        tx, ty = np.sum(W * b["a1"], -1), np.sum(W * b["a2"], -1)
        errs.append(max(np.abs(gx - tx).max(), np.abs(gy - ty).max()))
    assert errs[1] < errs[0] / 3.5, errs


def _extended_duals(N, hw):
    """Points and dual basis vectors b1, b2 of the extended panel grid lines."""
    r = _extended_points(N, hw)
    import math
    hx = 0.5 * math.pi / N
    a = -0.25 * math.pi + hx * (np.arange(1 - hw, N + hw + 1) - 0.5)
    ta, tb = np.tan(a)[None, :], np.tan(a)[:, None]
    p15 = (1 + ta * ta + tb * tb) ** 1.5
    one = np.ones_like(p15)
    a1p = np.stack([(1 + ta * ta) * (1 + tb * tb) / p15, -ta * tb * (1 + ta * ta) / p15,
                    -ta * (1 + ta * ta) * one / p15], -1)
    a2p = np.stack([-ta * tb * (1 + tb * tb) / p15, (1 + ta * ta) * (1 + tb * tb) / p15,
                    -tb * (1 + tb * tb) * one / p15], -1)

    def face(v):
        return (v[None, ..., 0:1] * initial._EX[:, None, None, :] + v[None, ..., 1:2] * initial._EY[:, None, None, :]
                - v[None, ..., 2:3] * initial._EN[:, None, None, :])

    a1, a2 = face(a1p), face(a2p)
    g11, g12, g22 = (a1 * a1).sum(-1), (a1 * a2).sum(-1), (a2 * a2).sum(-1)
    det = g11 * g22 - g12 * g12
    b1 = (g22[..., None] * a1 - g12[..., None] * a2) / det[..., None]
    b2 = (-g12[..., None] * a1 + g11[..., None] * a2) / det[..., None]
    return r, b1, b2


@pytest.mark.parametrize("hw", [1, 2])
def test_ecs_a_vec_halo_is_fourth_order(hw):
    """The ecs_A_vec halo of the contravariant cross-polar flow against its
    exact contravariant components on the extended grid lines: fourth-order
    convergence, interior untouched."""
    from analytic_fields import cross_polar as _cross_polar
    errs = []
    for N in (24, 48):
        od = oracle.OracleCDomain(N, 42, radius=1.0)
        r, b1, b2 = _extended_duals(N, hw)
        Vx = _cross_polar(r)
        x, y, z = od.points("p")
        b = od.bases("p")
        Vp = _cross_polar(np.stack([x, y, z], -1))
        u, v = np.sum(Vp * b["b1"], -1), np.sum(Vp * b["b2"], -1)
        eu, ev = od.ecs_a_vec_halo(u, v, hw)
        assert np.array_equal(eu[:, hw:hw + N, hw:hw + N], u.reshape(6, N, N))
        errs.append(max(np.abs(eu - np.sum(Vx * b1, -1)).max(), np.abs(ev - np.sum(Vx * b2, -1)).max()))
    assert errs[0] < 1e-4 and errs[1] < errs[0] / 12.0, errs


# ------------------------------------------------------------------ ECS_xy
def _extended_nodes(N, hw):
    """Cartesian points of the extended node grid lines, (6, W, W, 3)."""
    import math
    hx = 0.5 * math.pi / N
    a = -0.25 * math.pi + hx * (np.arange(1 - hw, N + 2 + hw) - 1.0)
    ta, tb = np.tan(a)[None, :], np.tan(a)[:, None]
    sg = np.sqrt(1 + ta * ta + tb * tb)
    one = np.ones_like(sg)
    rp = np.stack([ta * one / sg, tb * one / sg, one / sg], -1)
    return (rp[None, ..., 0:1] * initial._EX[:, None, None, :] + rp[None, ..., 1:2] * initial._EY[:, None, None, :]
            - rp[None, ..., 2:3] * initial._EN[:, None, None, :])


@pytest.mark.parametrize("hw", [1, 3])
def test_ecs_xy_halo_is_fourth_order(hw):
    """The ECS_xy halo of the node (corner) mesh: every extended point of a
    smooth field, the synced panel edges included, converges at fourth order
    to the exact values (the reference's halo test prints these errors with
    no known answers)."""
    errs = []
    for N in (24, 48):
        od = oracle.OracleCDomain(N, 42, radius=1.0)
        r = _extended_nodes(N, hw)
        e = 0.0
        for lev in range(3):
            E = od.ecs_xy_halo(od.scalar_test_field("xyz", lev, "q"), hw)
            e = max(e, float(np.abs(E - r[..., lev]).max()))
        errs.append(e)
    assert errs[0] < 2e-6 and errs[1] < errs[0] / 12.0, errs


@pytest.mark.parametrize("order,rate", [(2, 1.9), (4, 3.5)])
def test_laplace_ch_halo_converges(order, rate):
    """laplace_ch_halo2 / laplace_ch_halo4 on z (an l = 1 field, eigenvalue
    -2/a^2): the 4th-order operator converges at second order (the halo's
    fourth-order error over h^2 at the edges), the 2nd-order one at first
    order (the reference's index pairing in one metric term)."""
    a = 6.371e6
    errs = []
    for N in (24, 48):
        od = oracle.OracleCDomain(N, 42)
        z = od.scalar_test_field("xyz", 2, "q")
        errs.append(float(np.abs(od.laplace_ch(z, order) - (-2 / a ** 2) * z).max() * a ** 2 / 2))
    assert errs[0] / errs[1] > rate, errs
    assert errs[0] < (0.03 if order == 2 else 1e-4)
