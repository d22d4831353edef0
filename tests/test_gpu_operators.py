"""GPU single operators and cube-edge syncs against the FP64 oracle, and the
reference's own known-answer test reproduced through the C-ABI.

Tolerances: FP64 operators agree with the oracle to 1e-13 relative (max-norm
over the field); the golden numbers must match to the 7 digits the
reference prints."""
import json
import os

import numpy as np
import pytest

import oracle
import cubedsphere_sbp_swm_gb300 as swm
from gpu_helpers import fmt7

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "diffops_ah_n32.json")))


def _ctx(N, order, **kw):
    return swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=order, radius=kw.get("radius", 1.0),
                                           omega=kw.get("omega", 1.0)))


def _field(op, a):
    f = op.create_field()
    f.upload(a)
    return f


def _maxrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("entry", [g for g in GOLDEN if g["kind"] in ("div", "grad", "curl")
                                   and g["sbp_order"] in (42, 43)], ids=lambda g: g["name"])
def test_golden_through_cabi(entry):
    """test_div / test_grad / test_curl (test_diffops_mod.f90) on the GPU."""
    N, order, kind = entry["N"], entry["sbp_order"], entry["kind"]
    od = oracle.OracleDomain(N, order, radius=1.0, omega=1.0)
    J = od.geometry()["J"]
    hx2 = ((np.pi / 2) / N) ** 2
    op = _ctx(N, order)
    out = []
    if kind in ("div", "curl"):
        fields = (("solid_rotation", True, None), ("cross_polar", True, "cross_polar_div")) \
            if kind == "div" else (("vsh_curl_free_10", False, None),
                                   ("cross_polar", False, "cross_polar_zeta"))
        for fname, contra, truth in fields:
            mx, l2 = 0.0, 0.0
            for lev in range(3):
                u, v = od.vector_test_field(fname, lev, contravariant=contra)
                res = op.create_field()
                if kind == "div":
                    op.calc_div(res, _field(op, u), _field(op, v))
                else:
                    op.calc_curl(res, _field(op, u), _field(op, v))
                r = res.download()
                if truth:
                    r = r - od.scalar_test_field(truth, lev)
                mx = max(mx, float(np.max(np.abs(r))))
                l2 += float(np.sum(r * r * J * hx2))
            out += [mx, np.sqrt(l2)]
    else:
        mxs, l2s = [0.0, 0.0], [0.0, 0.0]
        for lev in range(3):
            f = od.scalar_test_field("xyz", lev)
            tx, ty = od.vector_test_field("xyz_grad", lev, contravariant=False)
            gx, gy = op.create_field(), op.create_field()
            op.calc_grad(gx, gy, _field(op, f))
            for k, (g, t) in enumerate(((gx.download(), tx), (gy.download(), ty))):
                e = g - t
                mxs[k] = max(mxs[k], float(np.max(np.abs(e))))
                l2s[k] += float(np.sum(e * e * J * hx2))
        out = [mxs[0] + mxs[1], np.sqrt(l2s[0]) + np.sqrt(l2s[1])]
    for g, w in zip(out, entry["values"]):
        assert fmt7(g) == fmt7(w), f"{entry['name']}: {g!r} vs {w!r}"


@pytest.fixture(scope="module", params=[42, 63])
def pair(request):
    order = request.param
    N = 40
    od = oracle.OracleDomain(N, order)
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=order))
    rng = np.random.default_rng(order)
    from cubedsphere_sbp_swm_gb300 import initial
    h, u, v, _ = initial.balanced_zonal(N, 3, 12)
    return od, op, rng, (h, u, v)


def test_grad_div_curl_match_oracle(pair):
    od, op, rng, (h, u, v) = pair
    f = h + 50.0 * rng.standard_normal(h.shape)
    gx, gy = op.create_field(), op.create_field()
    op.calc_grad(gx, gy, _field(op, f))
    ox, oy = od.grad(f)
    assert _maxrel(gx.download(), ox) < 1e-13 and _maxrel(gy.download(), oy) < 1e-13
    d = op.create_field()
    op.calc_div(d, _field(op, u), _field(op, v))
    assert _maxrel(d.download(), od.div(u, v)) < 1e-12
    c = op.create_field()
    op.calc_curl(c, _field(op, u), _field(op, v))
    assert _maxrel(c.download(), od.curl(u, v)) < 1e-12


def test_syncs_match_oracle(pair):
    od, op, rng, _ = pair
    a = rng.standard_normal((6, op.n, op.n))
    b = rng.standard_normal((6, op.n, op.n))
    fa = _field(op, a)
    swm.create_halo_procedure(op, "Ah_scalar_sync").get_halo_scalar(fa)
    assert np.max(np.abs(fa.download() - od.sync_scalar(a))) < 1e-15
    fa, fb = _field(op, a), _field(op, b)
    swm.create_vector_halo_procedure(op, "ecs_Ah_vec_sync_covariant").get_halo_vector(fa, fb)
    ox, oy = od.sync_vector_cov(a, b)
    assert np.max(np.abs(fa.download() - ox)) < 1e-14
    assert np.max(np.abs(fb.download() - oy)) < 1e-14


def test_pointwise_operators_match_oracle(pair):
    od, op, rng, (h, u, v) = pair
    ut, vt = op.create_field(), op.create_field()
    fu, fv, fh = _field(op, u), _field(op, v), _field(op, h)
    op.co2contra(ut, vt, fu, fv)
    out, ovt = od.co2contra(u, v)
    assert _maxrel(ut.download(), out) < 1e-15 and _maxrel(vt.download(), ovt) < 1e-15
    hu, hv = op.create_field(), op.create_field()
    op.massflux(hu, hv, fh, ut, vt)
    assert _maxrel(hu.download(), h * out) < 1e-15
    curl = od.curl(u, v)
    cu, cv = op.create_field(), op.create_field()
    op.calc_coriolis_vec_inv(cu, cv, hu, hv, fh, _field(op, curl))
    ocu, ocv = od.coriolis(h * out, h * ovt, h, curl)
    assert _maxrel(cu.download(), ocu) < 1e-14 and _maxrel(cv.download(), ocv) < 1e-14


def test_quadrature_mass_matches_oracle(pair):
    od, op, rng, (h, u, v) = pair
    m = op.quadrature_mass(_field(op, h))
    assert abs(m - od.mass(h)) / abs(od.mass(h)) < 1e-13
