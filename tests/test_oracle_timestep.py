"""The workloads' own time steps against the RK4 stability limit, shown with
the FP64 oracle itself (the reference arithmetic, rk4_mod.f90:20-42 over
operator_swm_mod.f90:61-113, no hyperdiffusion).

The Courant number c*dt/(a*hx), c = sqrt(g*5960 m) ~ 242 m/s, is 1.11 at
N=384, dt=120 s and at N=1024, dt=45 s, and 1.04 at N=48, dt=900 s: the
undiffused scheme turns non-finite there.  Courant 0.84 (N=384, 90 s), 0.74
(N=1024, 30 s) and 0.70 (N=48, 600 s), the time steps the accuracy runs use
instead, stay finite with the height deviation of a balanced flow."""
import os

import numpy as np
import pytest

import oracle
from cubedsphere_sbp_swm_gb300 import initial


def _run(od, state, dt, nsteps):
    h, u, v = (a.copy() for a in state)
    for k in range(nsteps):
        h, u, v = od.rk4(h, u, v, dt, 1)
        if not np.all(np.isfinite(h)):
            return k + 1, None
    return None, (h, u, v)


@pytest.fixture(autouse=True)
def _threads():
    oracle.set_threads(os.cpu_count() or 1)
    yield
    oracle.set_threads(1)


def test_n48_workload_dt_is_unstable_and_600s_is_not():
    h, u, v, _ = initial.config_state(1)
    od = oracle.OracleDomain(48, 42)
    bad, _ = _run(od, (h, u, v), 900.0, 640)          # 160 simulated hours
    assert bad is not None and bad > 96, bad           # after the 1-day run, before 160 h
    bad, out = _run(od, (h, u, v), 600.0, 1440)        # 10 simulated days
    assert bad is None
    assert np.max(np.abs(out[0] - h)) < 100.0


def test_n384_workload_dt_is_unstable_and_90s_is_not():
    h, u, v, _ = initial.config_state(2)
    od = oracle.OracleDomain(384, 42)
    bad, _ = _run(od, (h, u, v), 120.0, 60)            # 2 simulated hours
    assert bad is not None, "the N=384 state stayed finite at dt = 120 s"
    bad, out = _run(od, (h, u, v), 90.0, 120)          # 3 simulated hours
    assert bad is None
    assert np.max(np.abs(out[0] - h)) < 100.0


def test_n1024_d63_workload_dt_is_unstable_and_30s_is_not():
    """The large instance: Courant 1.11 at dt = 45 s (non-finite within 20
    simulated minutes), 0.74 at dt = 30 s."""
    h, u, v, _ = initial.config_state(5)
    od = oracle.OracleDomain(1024, 63)
    bad, _ = _run(od, (h, u, v), 45.0, 27)             # 20 simulated minutes
    assert bad is not None, "the N=1024 state stayed finite at dt = 45 s"
    bad, out = _run(od, (h, u, v), 30.0, 40)           # 20 simulated minutes
    assert bad is None
    assert np.max(np.abs(out[0] - h)) < 100.0
