"""Parity at the benchmarked configurations and for every SBP order.

The FP64 plain path against the FP64 oracle:
* one RK4 step of the N=384 SBP 4/2 workload (balanced zonal flow, degree
  <= 64 perturbation, dt = 120 s) and of the N=1024 SBP 6/3 workload (the
  barotropically unstable jet, dt = 45 s): the state within 1e-12 relative
  L2 (J-weighted, vec_math_mod.f90:50-90) and the step's increment within
  1e-9 (the increment is the state difference of two O(1e3) fields, which
  costs about four digits);
* 96 steps of SBP 6/3 at N=64 within 96 x 1e-12.

The FP32 fused form against the FP64 oracle for SBP 4/2, 4/3 and 6/3, one
step and 96 steps: h, u and v within 1e-5 relative L2, mass drift within
1e-6 of the oracle's; and one step of each benchmarked configuration: the
state within 1e-6 (measured: h 3e-8, u and v 3e-7), and the step's
increment within 0.1, a check of its direction only.  The stage inputs of
the FP32 form carry the high part of the state, and in these nearly
balanced flows h (about 6000 m, FP32 ulp 5e-4 m) moves by a few ulp per
step, so its increment is resolved to a few percent (measured: 3.6% at
N=384, 1.5% at N=1024; u and v 0.2-0.3%).  The compensated pair keeps what
the stages cannot resolve, which the state bound checks.
"""
import os

import numpy as np
import pytest

import oracle
import cubedsphere_sbp_swm_gb300 as swm
from cubedsphere_sbp_swm_gb300 import initial
from gpu_helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL_STEP = 1e-12
TOL_INCREMENT = 1e-9
TOL_FP32 = 1e-5


def _gpu_run(N, order, prec, state, dt, nsteps):
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=order, precision=prec))
    s = op.create_stvec()
    s.upload(*state)
    swm.RK4().step(s, op, dt, nsteps)
    out = s.download()
    del s, op
    return out


@pytest.mark.parametrize("cfg", [2, 5], ids=["n384_d42_dt120", "n1024_d63_dt45"])
def test_rk4_fp64_one_step_at_bench_config(cfg):
    c = initial.CONFIGS[cfg]
    N, order, dt = c["N"], c["sbp_order"], c["dt"]
    h, u, v, _ = initial.config_state(cfg)
    oracle.set_threads(os.cpu_count() or 1)
    od = oracle.OracleDomain(N, order)
    J = initial.ecs_geometry(N)["J"]
    got = _gpu_run(N, order, "fp64", (h, u, v), dt, 1)
    ref = od.rk4(h, u, v, dt, 1)
    for name, g, r, x0 in zip("huv", got, ref, (h, u, v)):
        e = rel_l2(g, r, J)
        assert e < TOL_STEP, (name, e)
        ei = rel_l2(g - x0, r - x0, J)
        assert ei < TOL_INCREMENT, (name, ei)


def test_rk4_fp64_d63_96_steps():
    N, dt = 64, 300.0
    h, u, v, _ = initial.balanced_zonal(N, 11, 16)
    od = oracle.OracleDomain(N, 63)
    J = od.geometry()["J"]
    got = _gpu_run(N, 63, "fp64", (h, u, v), dt, 96)
    ref = od.rk4(h, u, v, dt, 96)
    errs = [rel_l2(g, r, J) for g, r in zip(got, ref)]
    assert max(errs) < 96 * TOL_STEP, errs
    assert all(np.isfinite(g).all() for g in got)


@pytest.mark.parametrize("order,N", [(42, 48), (43, 40), (63, 48)])
@pytest.mark.parametrize("nsteps", [1, 96])
def test_rk4_fp32_fused_vs_fp64_oracle(order, N, nsteps):
    dt = 300.0
    h, u, v, _ = initial.balanced_zonal(N, 5, 16)
    od = oracle.OracleDomain(N, order)
    J = od.geometry()["J"]
    gh, gu, gv = _gpu_run(N, order, "fp32", (h, u, v), dt, nsteps)
    oh, ou, ov = od.rk4(h, u, v, dt, nsteps)
    errs = {k: rel_l2(a, b, J) for k, a, b in (("h", gh, oh), ("u", gu, ou), ("v", gv, ov))}
    assert max(errs.values()) < TOL_FP32, errs
    drift = abs(od.mass(gh) - od.mass(oh)) / od.mass(oh)
    assert drift < 1e-6, drift


@pytest.mark.parametrize("cfg", [2, 5], ids=["n384_d42_dt120", "n1024_d63_dt45"])
def test_rk4_fp32_one_step_at_bench_config(cfg):
    c = initial.CONFIGS[cfg]
    N, order, dt = c["N"], c["sbp_order"], c["dt"]
    h, u, v, _ = initial.config_state(cfg)
    oracle.set_threads(os.cpu_count() or 1)
    od = oracle.OracleDomain(N, order)
    J = initial.ecs_geometry(N)["J"]
    got = _gpu_run(N, order, "fp32", (h, u, v), dt, 1)
    ref = od.rk4(h, u, v, dt, 1)
    for name, g, r, x0 in zip("huv", got, ref, (h, u, v)):
        e = rel_l2(g, r, J)
        assert e < 1e-6, (name, e)
        ei = rel_l2(g - x0, r - x0, J)
        assert ei < 0.1, (name, ei)
