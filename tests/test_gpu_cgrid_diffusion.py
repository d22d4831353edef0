"""The C-grid hyperdiffusion on the GPU through the C-ABI, against the FP64
oracle: operator_swm_diff_t with the &shallow_water_model_c names
(hordiff_c_biharm_div / _curl / _curl_div for the velocity, hordiff_scalar_C
for h; hordiff_factory_mod.f90:19-36, 53-139, 196-247), its two operators
that the model's right-hand side does not use (grad_perp_c_sbp and the
contra2co transform of co2contra_c_sbp*_new), the explicit Euler diffusion
step and the drivers' step (RK4, then the diffusion step).

Tolerances: FP64 1e-12 relative L2 on operators and states (the tendencies
of a rough state are not cancellation-dominated); the FP32 form 1e-5 on
states (the bound of the RK4 step) and 1e-4 on the FP32 tendency of a rough
state.  The reference's contra2co known answers are pinned through the GPU
operators in test_gpu_cgrid.py.
"""
import numpy as np
import pytest

import cubedsphere_sbp_swm_gb300 as swm
import oracle
from cubedsphere_sbp_swm_gb300 import initial

pytestmark = pytest.mark.gpu

UV_NAMES = ("hordiff_c_biharm_div", "hordiff_c_biharm_curl", "hordiff_c_biharm_curl_div")


def c_op(N, order, **kw):
    return swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=order, names=swm.c_grid_names(order), **kw))


def field(op, mesh, a=None):
    f = op.create_field(mesh)
    if a is not None:
        f.upload(a)
    return f


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _rough_state(N, seed):
    """The seeded balanced flow plus grid-scale noise: the scales the
    hyperdiffusion acts on."""
    h, u, v, _ = initial.balanced_zonal_c(N, seed, 12)
    rng = np.random.default_rng(seed)
    return (h + 5.0 * rng.standard_normal(h.shape), u + rng.standard_normal(u.shape),
            v + rng.standard_normal(v.shape))


@pytest.mark.parametrize("order", [42, 21])
def test_grad_perp_and_contra2co_match_oracle(order):
    """Single operators on random inputs: a corner field that is not
    edge-synced exercises the SAT penalty of grad_perp on both sides."""
    N = 40
    op, od = c_op(N, order), oracle.OracleCDomain(N, order)
    rng = np.random.default_rng(order)
    w = rng.standard_normal(od.shapes["q"])
    gu, gv = field(op, "u"), field(op, "v")
    op.calc_grad_perp(gu, gv, field(op, "q", w))
    gu_o, gv_o = od.grad_perp(w)
    assert _rel(gu.download(), gu_o) < 1e-13 and _rel(gv.download(), gv_o) < 1e-13
    ut, vt = rng.standard_normal(od.shapes["u"]), rng.standard_normal(od.shapes["v"])
    u, v = field(op, "u"), field(op, "v")
    op.contra2co(u, v, field(op, "u", ut), field(op, "v", vt))
    u_o, v_o = od.contra2co(ut, vt)
    assert _rel(u.download(), u_o) < 1e-13 and _rel(v.download(), v_o) < 1e-13


@pytest.mark.parametrize("uv_name", UV_NAMES)
@pytest.mark.parametrize("order", [42, 21])
def test_diffusion_tendency_matches_oracle(order, uv_name):
    N = 40
    op, od = c_op(N, order), oracle.OracleCDomain(N, order)
    dop = swm.OperatorSWMDiff(op, uv_name, 0.03, "hordiff_scalar_C", 0.02)
    h, u, v = _rough_state(N, 3)
    vin = op.create_stvec()
    vin.upload(h, u, v)
    vout = vin.create_similar()
    dop.apply(vout, vin)
    for a, b in zip(vout.download(), od.hordiff(h, u, v, uv_name, 0.03, 0.02)):
        assert _rel(a, b) < 1e-12, _rel(a, b)


@pytest.mark.parametrize("order,prec,tol", [(42, "fp64", 1e-12), (21, "fp64", 1e-12), (42, "fp32", 1e-5)])
def test_model_step_with_diffusion_matches_oracle(order, prec, tol):
    """The namelist's C-grid configuration (namelist_swm:80-102: the 4/2
    operators, hordiff_c_biharm_curl_div and hordiff_scalar_C at 0.03):
    twelve drivers' steps against the oracle."""
    N, steps = 40, 12
    dt = 600.0 * 24 / N
    op, od = c_op(N, order, precision=prec), oracle.OracleCDomain(N, order)
    swm.OperatorSWMDiff(op)  # the namelist defaults of the C grid
    h, u, v = _rough_state(N, 7)
    s = op.create_stvec()
    s.upload(h, u, v)
    op.model_step(s, dt, steps)
    want = od.model_step(h, u, v, dt, steps, uv_name="hordiff_c_biharm_curl_div", uv_coeff=0.03, h_coeff=0.03)
    for a, b in zip(s.download(), want):
        assert _rel(a, b) < steps * tol, _rel(a, b)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_explicit_euler_diffusion_steps(prec, tol):
    """ExplicitEul1 with the diffusion operator: v0 += dt D(v0), three
    steps, against the oracle's tendencies applied in FP64."""
    N, dt = 32, 900.0
    op, od = c_op(N, 42, precision=prec), oracle.OracleCDomain(N, 42)
    dop = swm.OperatorSWMDiff(op, "hordiff_c_biharm_curl_div", 0.05, "hordiff_scalar_C", 0.04)
    h, u, v = _rough_state(N, 4)
    s = op.create_stvec()
    s.upload(h, u, v)
    swm.ExplicitEul1().step(s, dop, dt, 3)
    x = [h.copy(), u.copy(), v.copy()]
    for _ in range(3):
        t = od.hordiff(*x, "hordiff_c_biharm_curl_div", 0.05, 0.04)
        x = [a + dt * b for a, b in zip(x, t)]
    for a, b in zip(s.download(), x):
        assert _rel(a, b) < tol, _rel(a, b)


def test_fp32_diffusion_tendency():
    N = 32
    op, od = c_op(N, 42, precision="fp32"), oracle.OracleCDomain(N, 42)
    dop = swm.OperatorSWMDiff(op)
    h, u, v = _rough_state(N, 5)
    vin = op.create_stvec()
    vin.upload(h, u, v)
    vout = vin.create_similar()
    dop.apply(vout, vin)
    for a, b in zip(vout.download(), od.hordiff(h, u, v)):
        assert _rel(a, b) < 1e-4, _rel(a, b)


def test_diffusion_names_are_per_grid():
    """The C-grid names are refused on the Ah grid and the Ah-grid names on
    the C grid (SWM_E_UNSUPPORTED, no device work); grad_perp and contra2co
    exist on the C grid only."""
    cop = c_op(24, 42)
    with pytest.raises(swm.SwmError) as e:
        swm.OperatorSWMDiff(cop, "hordiff_vec_xyz_Ah_sbp_42_narrow", 0.03, "hordiff_scalar_C", 0.03)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED
    with pytest.raises(swm.SwmError) as e:
        swm.OperatorSWMDiff(cop, "hordiff_c_biharm_curl_div", 0.03, "hordiff_scalar_Ah_sbp_42_narrow", 0.03)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED
    aop = swm.OperatorSWM(swm.ModelConfig(N=24))
    with pytest.raises(swm.SwmError) as e:
        swm.OperatorSWMDiff(aop, "hordiff_c_biharm_curl_div", 0.03, "hordiff_scalar_C", 0.03)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED
    f = aop.create_field()
    with pytest.raises(swm.SwmError) as e:
        aop.calc_grad_perp(f, f, f)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED
    with pytest.raises(swm.SwmError) as e:
        aop.contra2co(f, f, f, f)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED
    # a diffusion step before any configuration is an argument error
    s = cop.create_stvec()
    with pytest.raises(swm.SwmError) as e:
        cop._check(cop._L.swm_diffusion_step(cop._h, s._h, 1.0, 1))
    assert e.value.code == swm._abi.SWM_E_INVALID


def test_co2contra_new_name_is_the_same_operator():
    """A namelist may name co2contra_c_sbpNN_new as the model's co2contra
    operator: the same interpolate / J Qi12 / interpolate back / divide by J
    map, so the context and its RK4 step are identical."""
    N = 24
    names = swm.c_grid_names(42)
    names["co2contra_op_name"] = "co2contra_c_sbp42_new"
    a = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, names=names))
    b = c_op(N, 42)
    h, u, v = _rough_state(N, 2)
    sa, sb = a.create_stvec(), b.create_stvec()
    sa.upload(h, u, v)
    sb.upload(h, u, v)
    swm.RK4().step(sa, a, 600.0, 2)
    swm.RK4().step(sb, b, 600.0, 2)
    for x, y in zip(sa.download(), sb.download()):
        assert np.array_equal(x, y)
