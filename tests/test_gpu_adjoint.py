"""Tangent-linear (TL) and adjoint (AD) of the FP64 model and the
checkpointed gradient of an RK4 trajectory.

The reference has no adjoint, so correctness is shown the standard way:
- dot-product tests <TL dx, l> = <dx, AD l> for the model operator, one RK4
  step and a whole trajectory: relative gap <= 1e-10 (the bar for FP64; the
  observed gaps are ~1e-14);
- TL against central finite differences of the forward operator (F is
  quadratic in the state, so the central difference is exact up to
  round-off): relative L2 <= 1e-7;
- the gradient of J = 1/2 sum w (h_T - h_obs)^2 (SBP quadrature weights w)
  against central finite differences of J along seeded random directions:
  relative gap <= 1e-5 at eps = 1e-6;
- the checkpointed sweep against the plain reverse sweep over stored states;
- the torch.autograd path against the direct one."""
import numpy as np
import pytest

import cubedsphere_sbp_swm_gb300 as swm
from cubedsphere_sbp_swm_gb300 import adjoint as ad
from cubedsphere_sbp_swm_gb300 import initial

pytestmark = pytest.mark.gpu

N, T, DT = 32, 20, 900.0          # Courant 0.70


def _dot(a, b):
    return float(sum(np.sum(x * y) for x, y in zip(a, b)))


def _stvec(op, arrs):
    s = op.create_stvec()
    s.upload(*arrs)
    return s


def _rand(rng, op, scale=(1.0, 1.0, 1.0)):
    return tuple(scale[k] * rng.standard_normal(op.shape) for k in range(3))


@pytest.fixture(scope="module", params=[42, 63])
def setup(request):
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=request.param))
    x0 = initial.balanced_zonal(N, 3, 16)[:3]
    return op, x0


def test_operator_dot_product(setup):
    op, x0 = setup
    rng = np.random.default_rng(11)
    y = _stvec(op, x0)
    dx, lk = _rand(rng, op), _rand(rng, op)
    dk, lx = op.create_stvec(), op.create_stvec()
    ad.apply_tl(op, y, _stvec(op, dx), dk)
    ad.apply_ad(op, y, _stvec(op, lk), lx)
    a, b = _dot(dk.download(), lk), _dot(dx, lx.download())
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b))


def test_tangent_linear_matches_central_differences(setup):
    op, x0 = setup
    rng = np.random.default_rng(12)
    dx = _rand(rng, op, (1.0, 0.1, 0.1))
    eps = 1e-3
    y = _stvec(op, x0)
    dk = op.create_stvec()
    ad.apply_tl(op, y, _stvec(op, dx), dk)
    fp, fm = op.create_stvec(), op.create_stvec()
    op.apply(fp, _stvec(op, [a + eps * d for a, d in zip(x0, dx)]))
    op.apply(fm, _stvec(op, [a - eps * d for a, d in zip(x0, dx)]))
    fd = [(p - m) / (2 * eps) for p, m in zip(fp.download(), fm.download())]
    for got, ref in zip(dk.download(), fd):
        assert np.linalg.norm(got - ref) <= 1e-7 * np.linalg.norm(ref)


def test_rk4_step_dot_product(setup):
    op, x0 = setup
    rng = np.random.default_rng(13)
    x = _stvec(op, x0)
    dx, lam = _rand(rng, op), _rand(rng, op)
    sdx, slam = _stvec(op, dx), _stvec(op, lam)
    ad.rk4_tl(op, x, sdx, DT)
    ad.rk4_ad(op, x, slam, DT)
    a, b = _dot(sdx.download(), lam), _dot(dx, slam.download())
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b))


def _trajectory(op, x0, steps):
    """x_0 .. x_steps by swm_rk4_step."""
    s = _stvec(op, x0)
    xs = [x0]
    for _ in range(steps):
        swm.RK4().step(s, op, DT, 1)
        xs.append(s.download())
    return xs


@pytest.mark.parametrize("nsnap", [1, 4, 16, 20])
def test_checkpointed_gradient_matches_stored_sweep(setup, nsnap):
    op, x0 = setup
    rng = np.random.default_rng(14)
    xs = _trajectory(op, x0, T)
    lamT = _rand(rng, op)
    # plain reverse sweep over stored states
    lam = _stvec(op, lamT)
    for n in range(T - 1, -1, -1):
        ad.rk4_ad(op, _stvec(op, xs[n]), lam, DT)
    ref = lam.download()
    run = ad.CheckpointedRK4(op, DT, T, nsnap)
    xT = op.create_stvec()
    run.forward(_stvec(op, x0), xT)
    for a, b in zip(xT.download(), xs[T]):
        assert np.array_equal(a, b)
    lam2 = _stvec(op, lamT)
    run.backward(lam2)
    for a, b in zip(lam2.download(), ref):
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
    c = run.counts()
    assert c["adjoint_steps"] == T
    assert c["forward_steps"] == c["planned_forward_steps"]
    if nsnap >= T:
        assert c["forward_steps"] == T          # every step once
    else:
        assert c["forward_steps"] > T


def test_trajectory_dot_product(setup):
    op, x0 = setup
    rng = np.random.default_rng(15)
    xs = _trajectory(op, x0, T)
    dx0, lamT = _rand(rng, op), _rand(rng, op)
    d = _stvec(op, dx0)
    for n in range(T):
        ad.rk4_tl(op, _stvec(op, xs[n]), d, DT)
    run = ad.CheckpointedRK4(op, DT, T, 4)
    run.forward(_stvec(op, x0), op.create_stvec())
    lam = _stvec(op, lamT)
    run.backward(lam)
    a, b = _dot(d.download(), lamT), _dot(dx0, lam.download())
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b))


def _cost(op, x0, w, hobs):
    s = _stvec(op, x0)
    swm.RK4().step(s, op, DT, T)
    h = s.download()[0]
    return 0.5 * float(np.sum(w * (h - hobs) ** 2))


def test_gradient_matches_finite_differences(setup):
    op, x0 = setup
    w = ad.quadrature_weights(op)
    hobs = _trajectory(op, initial.balanced_zonal(N, 4, 16)[:3], T)[T][0]
    run = ad.CheckpointedRK4(op, DT, T, 16)
    xT = op.create_stvec()
    run.forward(_stvec(op, x0), xT)
    hT = xT.download()[0]
    lam = _stvec(op, (w * (hT - hobs), np.zeros(op.shape), np.zeros(op.shape)))
    run.backward(lam)
    grad = lam.download()
    eps = 1e-6
    for k in range(5):
        d = _rand(np.random.default_rng(5 + k), op)
        jp = _cost(op, [a + eps * b for a, b in zip(x0, d)], w, hobs)
        jm = _cost(op, [a - eps * b for a, b in zip(x0, d)], w, hobs)
        fd, an = (jp - jm) / (2 * eps), _dot(grad, d)
        assert abs(fd - an) <= 1e-5 * abs(an), (k, fd, an)


def test_torch_autograd_matches_direct(setup):
    torch = pytest.importorskip("torch")
    op, x0 = setup
    w = ad.quadrature_weights(op)
    hobs = _trajectory(op, initial.balanced_zonal(N, 4, 16)[:3], T)[T][0]
    run = ad.CheckpointedRK4(op, DT, T, 4)
    dev = torch.device("cuda", 0)
    x = torch.tensor(np.stack(x0), device=dev, requires_grad=True)
    xT = ad.trajectory(x, run)
    wt, ht = torch.tensor(w, device=dev), torch.tensor(hobs, device=dev)
    loss = 0.5 * torch.sum(wt * (xT[0] - ht) ** 2)
    loss.backward()
    # direct
    run2 = ad.CheckpointedRK4(op, DT, T, 4)
    sT = op.create_stvec()
    run2.forward(_stvec(op, x0), sT)
    hT = sT.download()[0]
    assert np.array_equal(xT[0].detach().cpu().numpy(), hT)
    lam = _stvec(op, (w * (hT - hobs), np.zeros(op.shape), np.zeros(op.shape)))
    run2.backward(lam)
    for a, b in zip(x.grad.cpu().numpy(), lam.download()):
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))


def test_fp32_context_rejects_the_tangent_linear_model():
    op = swm.OperatorSWM(swm.ModelConfig(N=N, precision="fp32"))
    s = op.create_stvec()
    with pytest.raises(swm.SwmError) as e:
        ad.rk4_tl(op, s, op.create_stvec(), DT)
    assert e.value.code == swm._abi.SWM_E_UNSUPPORTED


def _rel(a, b):
    return float(np.sqrt(sum(np.sum((x - y) ** 2) for x, y in zip(a, b)) /
                         sum(np.sum(y * y) for y in b)))


@pytest.mark.parametrize("order", [42, 63])
def test_fp32_adjoint_step_matches_fp64(order):
    """One FP32 adjoint step against the FP64 one on the same base state and
    cotangent: relative L2 <= 1e-4 (FP32 stencil arithmetic)."""
    x0 = initial.balanced_zonal(N, 3, 16)[:3]
    rng = np.random.default_rng(21)
    lam = tuple(rng.standard_normal((6, N + 1, N + 1)) for _ in range(3))
    out = {}
    for prec in ("fp64", "fp32"):
        op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=order, precision=prec))
        lx = _stvec(op, lam)
        ad.rk4_ad(op, _stvec(op, x0), lx, DT)
        out[prec] = lx.download()
    assert _rel(out["fp32"], out["fp64"]) <= 1e-4


def test_fp32_checkpointed_gradient_matches_fp64():
    """Gradient of J over 20 steps with 4 snapshots, FP32 against FP64:
    relative L2 of the gradient <= 1e-3."""
    x0 = initial.balanced_zonal(N, 3, 16)[:3]
    grads = {}
    for prec in ("fp64", "fp32"):
        op = swm.OperatorSWM(swm.ModelConfig(N=N, precision=prec))
        w = ad.quadrature_weights(op)
        hobs = _trajectory(op, initial.balanced_zonal(N, 4, 16)[:3], T)[T][0]
        run = ad.CheckpointedRK4(op, DT, T, 4)
        xT = op.create_stvec()
        run.forward(_stvec(op, x0), xT)
        hT = xT.download()[0]
        lam = _stvec(op, (w * (hT - hobs), np.zeros(op.shape), np.zeros(op.shape)))
        run.backward(lam)
        grads[prec] = lam.download()
        assert run.counts()["adjoint_steps"] == T
    assert _rel(grads["fp32"], grads["fp64"]) <= 1e-3
