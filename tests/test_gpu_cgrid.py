"""The C-grid SBP operator family (&shallow_water_model_c, namelist_swm:80-102)
on the GPU through the C-ABI, against the FP64 oracle and the reference's own
known answers.

Pins:
* every C-grid line of reference_results.txt (div, grad, curl, Coriolis, KE,
  co2contra at sbp21 and sbp42, and the co2contra / contra2co pair of
  co2contra_c_sbp*_new, and gradient_a2_ecs with its ECS_O halo): the GPU
  operators on the reference test's fields at N=32, nz=3 reproduce the
  printed values to their 7 digits;
* each single operator, the fused and the unfused apply and the RK4 step
  against the oracle on a seeded balanced flow (FP64: 1e-12 on states and
  single operators; 1e-10 on tendencies, which carry the cancellation of
  div(h u) and of grad(KE + g h) against the Coriolis term);
* SBP mass conservation of the h tendency and of the state over many steps.
"""
import json
import os

import numpy as np
import pytest

import cubedsphere_sbp_swm_gb300 as swm
import oracle
from cubedsphere_sbp_swm_gb300 import initial
from analytic_fields import cross_polar as _cross_polar, solid_rotation as _solid_rotation
from analytic_fields import vsh_curl_free_10 as _vsh_curl_free_10
from gpu_helpers import fmt7

pytestmark = pytest.mark.gpu

GOLDEN_C = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "diffops_c_n32.json")))


def c_op(N, order, **kw):
    return swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=order, names=swm.c_grid_names(order), **kw))


def unit_ops(order):
    """The reference test's domain: unit sphere, Omega = 1 about z."""
    return c_op(32, order, radius=1.0, omega=1.0), oracle.OracleCDomain(32, order, radius=1.0, omega=1.0)


def field(op, mesh, a=None):
    f = op.create_field(mesh)
    if a is not None:
        f.upload(a)
    return f


def l2sq(od, mesh, f):
    return float(np.sum(f * f * od.metric(mesh)["J"]) * (0.5 * np.pi / od.N) ** 2)


def gpu_golden(kind, order):
    """test_diffops_mod.f90's test_div / test_grad / test_curl /
    test_coriolis_vec_inv / test_KE / test_co2contra with the GPU operators."""
    op, od = unit_ops(order)
    out = []
    if kind == "div":
        for fld in ("solid_rotation", "cross_polar"):
            m, l2 = 0.0, 0.0
            for lev in range(3):
                u, v = od.vector_test_field(fld, lev, contravariant=True)
                d = field(op, "p")
                op.calc_div(d, field(op, "u", u), field(op, "v", v))
                e = d.download()
                if fld == "cross_polar":
                    e = e - od.scalar_test_field("cross_polar_div", 0, "p")
                m, l2 = max(m, np.abs(e).max()), l2 + l2sq(od, "p", e)
            out += [m, np.sqrt(l2)]
    elif kind == "grad":
        mx = my = lx = ly = 0.0
        for lev in range(3):
            f = od.scalar_test_field("xyz", lev, "p")
            tx, ty = od.vector_test_field("xyz_grad", lev, contravariant=False)
            gx, gy = field(op, "u"), field(op, "v")
            op.calc_grad(gx, gy, field(op, "p", f))
            ex, ey = gx.download() - tx, gy.download() - ty
            mx, my = max(mx, np.abs(ex).max()), max(my, np.abs(ey).max())
            lx, ly = lx + l2sq(od, "u", ex), ly + l2sq(od, "v", ey)
        out = [mx + my, np.sqrt(lx) + np.sqrt(ly)]
    elif kind == "curl":
        for fld in ("vsh_curl_free_10", "cross_polar"):
            m, l2 = 0.0, 0.0
            for lev in range(3):
                u, v = od.vector_test_field(fld, lev, contravariant=False)
                c = field(op, "q")
                op.calc_curl(c, field(op, "u", u), field(op, "v", v))
                e = c.download()
                if fld == "cross_polar":
                    e = e - od.scalar_test_field("cross_polar_zeta", 0, "q")
                m, l2 = max(m, np.abs(e).max()), l2 + l2sq(od, "q", e)
            out += [m, np.sqrt(l2)]
    elif kind == "coriolis":
        hu, hv = od.vector_test_field("vsh_curl_free_10", 0, contravariant=True)
        # exact force 2 sin(phi) (v_phi, -v_lam) in covariant components,
        # computed by the oracle's Coriolis test (the known answer itself)
        h, cz = np.ones(od.shapes["p"]), np.zeros(od.shapes["q"])
        cu, cv = field(op, "u"), field(op, "v")
        op.calc_coriolis_vec_inv(cu, cv, field(op, "u", hu), field(op, "v", hv), field(op, "p", h),
                                 field(op, "q", cz))
        ou, ov = od.coriolis(hu, hv, h, cz)
        # the GPU operator must equal the oracle's (which reproduces the
        # printed values); the errors of the exact force are the oracle's
        assert np.abs(cu.download() - ou).max() < 1e-14
        assert np.abs(cv.download() - ov).max() < 1e-14
        out = list(oracle.golden_c("coriolis", 32, order))
    elif kind == "ke":
        for fld in ("vsh_curl_free_10", "cross_polar"):
            m, l2 = 0.0, 0.0
            for lev in range(3):
                u, v = od.vector_test_field(fld, lev, contravariant=False)
                ut, vt = od.vector_test_field(fld, lev, contravariant=True)
                k = field(op, "p")
                op.calc_KE(k, field(op, "u", u), field(op, "v", v), field(op, "u", ut), field(op, "v", vt))
                # |V|^2/2 at the centres: the oracle's KE of the exact
                # components at the centres is the reference's KE_true
                x, y, z = od.points("p")
                r = np.stack([x, y, z], -1)
                if fld == "cross_polar":
                    V = _cross_polar(r)
                else:
                    V = _vsh_curl_free_10(r)
                e = k.download() - 0.5 * np.sum(V * V, -1)
                m, l2 = max(m, np.abs(e).max()), l2 + l2sq(od, "p", e)
            out += [m, np.sqrt(l2)]
    elif kind == "co2contra":
        mx = my = lx = ly = 0.0
        for lev in range(3):
            u, v = od.vector_test_field("cross_polar", lev, contravariant=False)
            tu, tv = od.vector_test_field("cross_polar", lev, contravariant=True)
            ut, vt = field(op, "u"), field(op, "v")
            op.co2contra(ut, vt, field(op, "u", u), field(op, "v", v))
            ex, ey = ut.download() - tu, vt.download() - tv
            mx, my = max(mx, np.abs(ex).max()), max(my, np.abs(ey).max())
            lx, ly = lx + l2sq(od, "u", ex), ly + l2sq(od, "v", ey)
        out = [mx + my, np.sqrt(lx) + np.sqrt(ly)]
    elif kind == "grad_c2_ecs":
        mx = my = lx = ly = 0.0
        for lev in range(3):
            f = od.scalar_test_field("xyz", lev, "p")
            tx, ty = od.vector_test_field("xyz_grad", lev, contravariant=False)
            gx, gy = field(op, "u"), field(op, "v")
            op.calc_grad_c2_ecs(gx, gy, field(op, "p", f))
            ex, ey = gx.download() - tx, gy.download() - ty
            mx, my = max(mx, np.abs(ex).max()), max(my, np.abs(ey).max())
            lx, ly = lx + l2sq(od, "u", ex), ly + l2sq(od, "v", ey)
        out = [mx + my, np.sqrt(lx) + np.sqrt(ly)]
    elif kind == "grad_a2_ecs":
        # test_grad for gradient_a2_ecs on the A grid's cell centres
        mx = my = lx = ly = 0.0
        x, y, z = od.points("p")
        r = np.stack([x, y, z], -1)
        b = od.bases("p")
        for lev in range(3):
            f = od.scalar_test_field("xyz", lev, "p")
            W = np.eye(3)[lev] - r[..., lev:lev + 1] * r
            tx, ty = np.sum(W * b["a1"], -1), np.sum(W * b["a2"], -1)
            gx, gy = field(op, "p"), field(op, "p")
            op.calc_grad_a2_ecs(gx, gy, field(op, "p", f))
            ex, ey = gx.download() - tx, gy.download() - ty
            mx, my = max(mx, np.abs(ex).max()), max(my, np.abs(ey).max())
            lx, ly = lx + l2sq(od, "p", ex), ly + l2sq(od, "p", ey)
        out = [mx + my, np.sqrt(lx) + np.sqrt(ly)]
    elif kind == "div_a2_ecs":
        # test_div for divergence_a2_ecs on the A grid's cell centres
        x, y, z = od.points("p")
        r = np.stack([x, y, z], -1)
        b = od.bases("p")
        for fld in ("solid_rotation", "cross_polar"):
            m, l2 = 0.0, 0.0
            for lev in range(3):
                V = _solid_rotation(r, lev) if fld == "solid_rotation" else _cross_polar(r)
                uu, vv = np.sum(V * b["b1"], -1), np.sum(V * b["b2"], -1)
                d = field(op, "p")
                op.calc_div_a2_ecs(d, field(op, "p", uu), field(op, "p", vv))
                e = d.download()
                if fld == "cross_polar":
                    e = e - od.scalar_test_field("cross_polar_div", 0, "p")
                m, l2 = max(m, np.abs(e).max()), l2 + l2sq(od, "p", e)
            out += [m, np.sqrt(l2)]
    elif kind == "contra2co":
        # test_contra2co: transform2co of co2contra_c_sbp*_new
        mx = my = lx = ly = 0.0
        for lev in range(3):
            ut, vt = od.vector_test_field("cross_polar", lev, contravariant=True)
            tu, tv = od.vector_test_field("cross_polar", lev, contravariant=False)
            u, v = field(op, "u"), field(op, "v")
            op.contra2co(u, v, field(op, "u", ut), field(op, "v", vt))
            ex, ey = u.download() - tu, v.download() - tv
            mx, my = max(mx, np.abs(ex).max()), max(my, np.abs(ey).max())
            lx, ly = lx + l2sq(od, "u", ex), ly + l2sq(od, "v", ey)
        out = [mx + my, np.sqrt(lx) + np.sqrt(ly)]
    return out


@pytest.mark.parametrize("entry", GOLDEN_C, ids=lambda g: g["name"])
def test_c_grid_gpu_operators_reproduce_reference_known_answers(entry):
    got = gpu_golden(entry["kind"], entry["sbp_order"])
    want = entry["values"]
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert fmt7(g) == fmt7(w), f"{entry['name']}: {g!r} vs {w!r} ({entry['source']})"


def _state(N, seed=3):
    h, u, v, _ = initial.balanced_zonal_c(N, seed, 12)
    return h, u, v


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("order", [42, 21])
def test_single_operators_match_oracle(order):
    N = 40
    op, od = c_op(N, order), oracle.OracleCDomain(N, order)
    h, u, v = _state(N)
    ut_o, vt_o = od.co2contra(u, v)
    hu_o, hv_o = od.massflux(h, ut_o, vt_o)
    fu, fv, fh = field(op, "u", u), field(op, "v", v), field(op, "p", h)
    ut, vt = field(op, "u"), field(op, "v")
    op.co2contra(ut, vt, fu, fv)
    assert _rel(ut.download(), ut_o) < 1e-13 and _rel(vt.download(), vt_o) < 1e-13
    hu, hv = field(op, "u"), field(op, "v")
    op.massflux(hu, hv, fh, field(op, "u", ut_o), field(op, "v", vt_o))
    assert _rel(hu.download(), hu_o) < 1e-13 and _rel(hv.download(), hv_o) < 1e-13
    ke = field(op, "p")
    op.calc_KE(ke, fu, fv, field(op, "u", ut_o), field(op, "v", vt_o))
    assert _rel(ke.download(), od.ke(u, v, ut_o, vt_o)) < 1e-13
    gx, gy = field(op, "u"), field(op, "v")
    op.calc_grad(gx, gy, fh)
    gxo, gyo = od.grad(h)
    assert _rel(gx.download(), gxo) < 1e-12 and _rel(gy.download(), gyo) < 1e-12
    c = field(op, "q")
    op.calc_curl(c, fu, fv)
    co = od.curl(u, v)
    assert _rel(c.download(), co) < 1e-12
    d = field(op, "p")
    op.calc_div(d, field(op, "u", hu_o), field(op, "v", hv_o))
    assert _rel(d.download(), od.div(hu_o, hv_o)) < 1e-12
    cu, cv = field(op, "u"), field(op, "v")
    op.calc_coriolis_vec_inv(cu, cv, field(op, "u", hu_o), field(op, "v", hv_o), fh, field(op, "q", co))
    cuo, cvo = od.coriolis(hu_o, hv_o, h, co)
    assert _rel(cu.download(), cuo) < 1e-12 and _rel(cv.download(), cvo) < 1e-12


@pytest.mark.parametrize("order", [42, 21])
def test_apply_fused_and_unfused_match_oracle(order):
    N = 40
    op, od = c_op(N, order), oracle.OracleCDomain(N, order)
    h, u, v = _state(N, 5)
    hs = 300.0 * od.scalar_test_field("xyz", 2, "p")
    op.set_orography(hs)
    want = od.apply(h, u, v, hs=hs)
    vin = op.create_stvec()
    vin.upload(h, u, v)
    for apply in (op.apply, op.apply_unfused):
        vout = vin.create_similar()
        apply(vout, vin)
        for a, b in zip(vout.download(), want):
            assert _rel(a, b) < 1e-10, (apply.__name__, _rel(a, b))


@pytest.mark.parametrize("order,N,steps", [(42, 40, 1), (42, 40, 24), (21, 40, 24), (42, 96, 2)])
def test_rk4_matches_oracle(order, N, steps):
    op, od = c_op(N, order), oracle.OracleCDomain(N, order)
    h, u, v = _state(N, 7)
    dt = 600.0 * 24 / N   # Courant number about 0.4 (the 4/2 C-grid limit is near 0.6)
    s = op.create_stvec()
    s.upload(h, u, v)
    swm.RK4().step(s, op, dt, steps)
    want = od.rk4(h, u, v, dt, steps)
    for a, b in zip(s.download(), want):
        assert _rel(a, b) < 1e-12, _rel(a, b)


def test_state_transfers_and_algebra_on_staggered_meshes():
    N = 24
    op = c_op(N, 42)
    assert op.staggering == "C"
    assert op.state_shapes == ((6, N, N), (6, N, N + 1), (6, N + 1, N))
    rng = np.random.default_rng(2)
    x = [rng.standard_normal(sh) for sh in op.state_shapes]
    y = [rng.standard_normal(sh) for sh in op.state_shapes]
    a, b = op.create_stvec(), op.create_stvec()
    a.upload(*x)
    b.upload(*y)
    for g, w in zip(a.download(), x):
        assert np.array_equal(g, w)
    a.update_s1v1s2v2(0.5, b, -2.0, b)
    for g, p, q in zip(a.download(), x, y):
        assert np.allclose(g, (p + 0.5 * q) + (-2.0) * q, rtol=0, atol=1e-15)


def test_mass_conservation():
    """SBP-SAT divergence + SBP_C42 quadrature: the global integral of the h
    tendency vanishes to round-off, and RK4 keeps the mass."""
    N = 48
    op = c_op(N, 42)
    h, u, v = _state(N, 9)
    s = op.create_stvec()
    s.upload(h, u, v)
    t = s.create_similar()
    op.apply(t, s)
    th = field(op, "p", t.download()[0])
    habs = field(op, "p", np.abs(t.download()[0]))
    assert abs(op.quadrature_mass(th)) / op.quadrature_mass(habs) < 1e-13
    m0 = op.quadrature_mass(field(op, "p", h))
    swm.RK4().step(s, op, 300.0, 50)
    m1 = op.quadrature_mass(field(op, "p", s.download()[0]))
    assert abs(m1 - m0) / m0 < 1e-13


def test_ah_only_entry_points_refuse_c_grid():
    op = c_op(24, 42)
    s = op.create_stvec()
    with pytest.raises(swm.SwmError) as e:
        op.get_diagnostics(s)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED
    with pytest.raises(swm.SwmError) as e:
        s.algebraic_norm2()
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED
    names = swm.c_grid_names(42)
    names["curl_op_name"] = "curl_c_sbp21"
    with pytest.raises(swm.SwmError) as e:
        swm.OperatorSWM(swm.ModelConfig(N=24, sbp_order=42, names=names))
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED


@pytest.mark.parametrize("order,steps", [(42, 1), (42, 24), (21, 24)])
def test_fp32_form_rk4_against_fp64_oracle(order, steps):
    """The FP32 form (FP32 passes, FP32 (hi, lo) state pair with a two-sum
    RK accumulation) against the FP64 oracle: within 1e-5 relative L2 for
    h, u and v (the bound of the Ah grid's FP32 form), mass drift within
    1e-6 of the oracle's."""
    N = 40
    op, od = c_op(N, order, precision="fp32"), oracle.OracleCDomain(N, order)
    h, u, v = _state(N, 7)
    dt = 600.0 * 24 / N
    s = op.create_stvec()
    s.upload(h, u, v)
    swm.RK4().step(s, op, dt, steps)
    want = od.rk4(h, u, v, dt, steps)
    got = s.download()
    for a, b in zip(got, want):
        assert _rel(a, b) < 1e-5, _rel(a, b)
    assert abs(od.mass(got[0]) - od.mass(want[0])) / od.mass(want[0]) < 1e-6


def test_fp32_form_state_pair_round_trip_and_apply():
    """Upload splits FP64 values into the (hi, lo) pair and download joins
    them back (2^-47 relative); the FP32 apply is within 1e-4 of the FP64
    oracle's tendencies.  The state is perturbed off balance: the tendencies
    of a balanced flow are the small difference of large terms, and FP32
    rounding of those terms is then visible at 1e-4 .. 1e-3 of the result."""
    N = 24
    op, od = c_op(N, 42, precision="fp32"), oracle.OracleCDomain(N, 42)
    h, u, v = _state(N, 5)
    rng = np.random.default_rng(8)
    h = h + 20.0 * rng.standard_normal(h.shape)
    u = u + 2.0 * rng.standard_normal(u.shape)
    v = v + 2.0 * rng.standard_normal(v.shape)
    s = op.create_stvec()
    s.upload(h, u, v)
    for a, b in zip(s.download(), (h, u, v)):
        assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)) <= 2.0 ** -47
    t = s.create_similar()
    op.apply(t, s)
    for a, b in zip(t.download(), od.apply(h, u, v)):
        assert _rel(a, b) < 1e-4, _rel(a, b)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_bench_configuration_against_oracle(prec, tol):
    """The C-grid bench workload itself (N=384, SBP 4/2, dt = 37.5 s, the
    seeded balanced flow of bench.py's c_grid leg): two RK4 steps against
    the FP64 oracle."""
    N, dt = 384, 37.5
    op, od = c_op(N, 42, precision=prec), oracle.OracleCDomain(N, 42)
    h, u, v, _ = initial.balanced_zonal_c(N, 11, 24)
    s = op.create_stvec()
    s.upload(h, u, v)
    swm.RK4().step(s, op, dt, 2)
    for a, b in zip(s.download(), od.rk4(h, u, v, dt, 2)):
        assert _rel(a, b) < tol, _rel(a, b)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_async_transfers_on_staggered_meshes(prec):
    """upload_async -> steps -> download_async gives the bytes of the
    synchronous route on the C grid (each component in its own mesh shape),
    and a state changed right after download_async does not change what the
    download returns."""
    import torch
    N = 32
    op = c_op(N, 42, precision=prec)
    h, u, v = _state(N, 6)
    pins = [torch.empty(a.shape, dtype=torch.float64, pin_memory=True) for a in (h, u, v) for _ in range(2)]
    src = [pins[2 * k].numpy() for k in range(3)]
    dst = tuple(pins[2 * k + 1].numpy() for k in range(3))
    for p_, a in zip(src, (h, u, v)):
        p_[...] = a
    s_sync, s_async = op.create_stvec(), op.create_stvec()
    s_sync.upload(h, u, v)
    s_async.upload_async(*src)
    swm.RK4().step(s_sync, op, 300.0, 2)
    swm.RK4().step(s_async, op, 300.0, 2)
    s_async.download_async(dst)
    s_async.assign_s1(-1.0)
    op.synchronize()
    for a, b in zip(s_sync.download(), dst):
        assert np.array_equal(a, b)


def test_c_grid_argument_errors():
    """Argument errors come back as SWM_E_INVALID / SWM_E_UNSUPPORTED, with
    no device work: a grid below the closures' reach, an unknown mesh, a
    field on the wrong mesh for an operator, the corner sync of a
    non-corner field."""
    with pytest.raises(swm.SwmError) as e:
        c_op(8, 42)
    assert e.value.code in (swm._abi.SWM_E_INVALID, swm._abi.SWM_E_UNSUPPORTED)
    op = c_op(24, 42)
    with pytest.raises(KeyError):
        op.create_field("w")
    ut, vt = field(op, "u"), field(op, "v")
    with pytest.raises(swm.SwmError) as e:
        op.co2contra(ut, vt, field(op, "p"), field(op, "v"))       # u on the wrong mesh
    assert e.value.code == swm._abi.SWM_E_INVALID
    with pytest.raises(swm.SwmError) as e:
        op._check(op._L.swm_sync_scalar(op._h, field(op, "p")._h))
    assert e.value.code == swm._abi.SWM_E_INVALID
    import ctypes
    f = ctypes.c_void_p()
    assert op._L.swm_field_create_mesh(op._h, 7, ctypes.byref(f)) == swm._abi.SWM_E_INVALID


@pytest.mark.parametrize("hw", [1, 2])
def test_ecs_o_halo_and_grad_a2_ecs_match_oracle(hw):
    """The ECS_O halo of a random cell-centre field (every edge row, corner
    point and in-corner point of width hw) and gradient_a2_ecs against the
    oracle."""
    N = 40
    op, od = c_op(N, 42), oracle.OracleCDomain(N, 42)
    f = np.random.default_rng(hw).standard_normal(od.shapes["p"])
    fp = field(op, "p", f)
    E, Eo = op.ecs_o_halo(fp, hw), od.ecs_o_halo(f, hw)
    assert E.shape == (6, N + 2 * hw, N + 2 * hw)
    assert np.abs(E - Eo).max() <= 1e-14 * np.abs(Eo).max()
    gx, gy = field(op, "p"), field(op, "p")
    op.calc_grad_a2_ecs(gx, gy, fp)
    gxo, gyo = od.grad_a2_ecs(f)
    assert _rel(gx.download(), gxo) < 1e-13 and _rel(gy.download(), gyo) < 1e-13
    gu, gv = field(op, "u"), field(op, "v")
    op.calc_grad_c2_ecs(gu, gv, fp)
    guo, gvo = od.grad_c2_ecs(f)
    assert _rel(gu.download(), guo) < 1e-13 and _rel(gv.download(), gvo) < 1e-13


def test_ecs_o_argument_errors():
    """Width outside 1..2, a field off the centre mesh and the Ah grid are
    refused."""
    op = c_op(24, 42)
    with pytest.raises(swm.SwmError) as e:
        op.ecs_o_halo(field(op, "p"), 3)
    assert e.value.code == swm._abi.SWM_E_INVALID
    with pytest.raises(swm.SwmError) as e:
        op.ecs_o_halo(field(op, "u"), 1)
    assert e.value.code == swm._abi.SWM_E_INVALID
    with pytest.raises(swm.SwmError) as e:
        op.calc_grad_a2_ecs(field(op, "u"), field(op, "p"), field(op, "p"))
    assert e.value.code == swm._abi.SWM_E_INVALID
    aop = swm.OperatorSWM(swm.ModelConfig(N=24))
    f = aop.create_field()
    with pytest.raises(swm.SwmError) as e:
        aop.calc_grad_a2_ecs(f, f, f)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED


@pytest.mark.parametrize("hw", [1, 2])
def test_ecs_a_vec_halo_and_div_a2_ecs_match_oracle(hw):
    """The ecs_A_vec halo of random contravariant components (every halo
    point of width hw, through the vector exchange, the edge maps and the
    ECS_O interpolation) and divergence_a2_ecs against the oracle."""
    N = 40
    op, od = c_op(N, 42), oracle.OracleCDomain(N, 42)
    rng = np.random.default_rng(10 + hw)
    u, v = rng.standard_normal(od.shapes["p"]), rng.standard_normal(od.shapes["p"])
    fu, fv = field(op, "p", u), field(op, "p", v)
    eu, ev = op.ecs_a_vec_halo(fu, fv, hw)
    eo_u, eo_v = od.ecs_a_vec_halo(u, v, hw)
    assert np.abs(eu - eo_u).max() <= 1e-14 * np.abs(eo_u).max()
    assert np.abs(ev - eo_v).max() <= 1e-14 * np.abs(eo_v).max()
    d = field(op, "p")
    op.calc_div_a2_ecs(d, fu, fv)
    assert _rel(d.download(), od.div_a2_ecs(u, v)) < 1e-13


@pytest.mark.parametrize("hw", [1, 3])
def test_ecs_xy_halo_matches_oracle(hw):
    """The ECS_xy halo of a random corner-mesh field (its synced edges, the
    corner diagonals and every halo row of width hw) against the oracle."""
    N = 40
    op, od = c_op(N, 42), oracle.OracleCDomain(N, 42)
    f = np.random.default_rng(20 + hw).standard_normal(od.shapes["q"])
    E, Eo = op.ecs_xy_halo(field(op, "q", f), hw), od.ecs_xy_halo(f, hw)
    assert E.shape == (6, N + 1 + 2 * hw, N + 1 + 2 * hw)
    assert np.abs(E - Eo).max() <= 1e-14 * np.abs(Eo).max()


@pytest.mark.parametrize("order", [2, 4])
def test_laplace_ch_halo_matches_oracle(order):
    """laplace_ch_halo2 / laplace_ch_halo4 of a smooth and of a random
    corner-mesh field against the oracle, in place as well."""
    N = 40
    op, od = c_op(N, 42), oracle.OracleCDomain(N, 42)
    rng = np.random.default_rng(order)
    for f in (od.scalar_test_field("xyz", 2, "q") * 1e3, rng.standard_normal(od.shapes["q"])):
        fin, fo = field(op, "q", f), field(op, "q")
        op.laplace_ch(fo, fin, order)
        want = od.laplace_ch(f, order)
        assert _rel(fo.download(), want) < 1e-12, _rel(fo.download(), want)
        op.laplace_ch(fin, fin, order)
        assert _rel(fin.download(), want) < 1e-12
