"""Ensembles: every member of a batched ensemble (uneven resolutions, own
seed and time step) advances exactly as the single-instance path advances
that member alone -- the same kernels and arithmetic, only the work split
and the launch differ -- for every tile shape the autotuner may pick, in
both precisions.  The autotuner leaves the member states as it found them.

Tolerance: bit-identical states (the per-node arithmetic does not depend on
the work split)."""
import numpy as np
import pytest

import cubedsphere_sbp_swm_gb300 as swm
from cubedsphere_sbp_swm_gb300 import initial

pytestmark = pytest.mark.gpu

MEMBERS = [32, 48, 40, 32, 64, 48]          # cells per panel edge, uneven


def _dt(N):
    return 600.0 * 48 / N                   # Courant 0.70 at every resolution


def _init():
    return [initial.balanced_zonal(N, 1000 + m, 16)[:3] for m, N in enumerate(MEMBERS)]


@pytest.fixture(scope="module")
def states():
    return _init()


@pytest.fixture(scope="module")
def single(states):
    """Each member stepped alone through swm_rk4_step: 3 steps, both forms."""
    out = {}
    for prec in ("fp32", "fp64"):
        res = []
        for N, st in zip(MEMBERS, states):
            op = swm.OperatorSWM(swm.ModelConfig(N=N, precision=prec))
            s = op.create_stvec()
            s.upload(*st)
            swm.RK4().step(s, op, _dt(N), 3)
            res.append(s.download())
        out[prec] = res
    return out


def _ensemble(prec, states):
    ens = swm.Ensemble(swm.ModelConfig(N=MEMBERS[0], precision=prec), MEMBERS,
                       [_dt(N) for N in MEMBERS])
    for m, st in enumerate(states):
        ens.upload(m, *st)
    return ens


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("seg_rows,persistent", [(0, True), (0, False), (16, True), (24, False),
                                                 (8, True)])
def test_members_match_single_instance(prec, seg_rows, persistent, states, single):
    ens = _ensemble(prec, states)
    ens.set_shape(seg_rows, 152 * 3 if persistent else 0)
    ens.step(3)
    ens.synchronize()
    for m in range(len(MEMBERS)):
        got = ens.download(m)
        for a, b in zip(got, single[prec][m]):
            assert np.array_equal(a, b), f"member {m} (N={MEMBERS[m]}) differs"


@pytest.mark.parametrize("width", [64, 96, 160, 192])
def test_member_widths_match_single_instance(width, states, single):
    ens = _ensemble("fp32", states)
    ens.set_width(width)
    assert ens.get_shape()["width"] == width
    ens.step(3)
    ens.synchronize()
    for m in range(len(MEMBERS)):
        for a, b in zip(ens.download(m), single["fp32"][m]):
            assert np.array_equal(a, b), f"member {m} (N={MEMBERS[m]}) differs at width {width}"


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_autotuner_keeps_states_and_picks_a_valid_shape(prec, states, single):
    ens = _ensemble(prec, states)
    before = [ens.download(m) for m in range(len(MEMBERS))]
    res = ens.tune(steps=2)
    assert res["ms_per_step"] > 0
    assert res["seg_rows"] >= 0 and res["grid"] >= 0
    # FP32: the TMA kernel's consumer widths; FP64: the plain kernel's one width
    assert res["width"] in ((64, 96, 128, 160, 192) if prec == "fp32" else (64,))
    sh = ens.get_shape()
    assert sh["seg_rows"] == res["seg_rows"] and sh["width"] == res["width"]
    for m in range(len(MEMBERS)):
        for a, b in zip(ens.download(m), before[m]):
            assert np.array_equal(a, b)
    ens.step(3)
    ens.synchronize()
    for m in range(len(MEMBERS)):
        for a, b in zip(ens.download(m), single[prec][m]):
            assert np.array_equal(a, b)


def test_member_diagnostics_and_access(states):
    ens = _ensemble("fp32", states)
    d = ens.get_diagnostics(2)
    assert set(d) == set(swm.DIAG_KEYS) and d["hmin"] > 0
    ctx, st = ens.member(1)
    assert ctx.value and st.value
    h, u, v = (np.ascontiguousarray(a) for a in states[0])
    ptr = [a.ctypes.data_as(swm._abi._D) for a in (h, u, v)]
    rc = ens._L.swm_ensemble_upload(ens._h, len(MEMBERS), *ptr)     # no such member
    assert rc == swm._abi.SWM_E_INVALID
    assert b"out of range" in ens._L.swm_ensemble_last_error(ens._h)


def test_wide_members_match_single_instance():
    """Members whose field pitch holds the widest TMA box of width 96
    (N >= 99): the ensemble launches the compile-time box kernel for all of
    them and still matches each member stepped alone."""
    wide = [128, 160, 144]
    sts = [initial.balanced_zonal(N, 2000 + m, 16)[:3] for m, N in enumerate(wide)]
    ref = []
    for N, st in zip(wide, sts):
        op = swm.OperatorSWM(swm.ModelConfig(N=N, precision="fp32"))
        op.set_stage_shape(96, 0, 0, "widest")
        s = op.create_stvec()
        s.upload(*st)
        swm.RK4().step(s, op, _dt(N), 2)
        ref.append(s.download())
    ens = swm.Ensemble(swm.ModelConfig(N=wide[0], precision="fp32"), wide, [_dt(N) for N in wide])
    for m, st in enumerate(sts):
        ens.upload(m, *st)
    ens.set_width(96)
    ens.step(2)
    ens.synchronize()
    for m in range(len(wide)):
        for a, b in zip(ens.download(m), ref[m]):
            assert np.array_equal(a, b), f"member {m} (N={wide[m]}) differs"
