"""swm_sync_scalar_static (the scalar cube-edge sync whose scratch is a fixed
array in the library's device image) against swm_sync_scalar, called through
the C-ABI.  Collected last so that it also runs after every other test; it
passes in a fresh process too, where its first call does the per-device
scratch look-up.

Tolerance: the cube-edge syncs agree with the oracle to 1e-15 absolute on
unit-variance fields; both entry points run the same arithmetic."""
import ctypes

import numpy as np
import pytest

import cubedsphere_sbp_swm_gb300 as swm

pytestmark = pytest.mark.gpu

TOL = 1e-15


def _op(N, order=42):
    return swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=order, radius=1.0, omega=1.0))


def _field(op, a):
    f = op.create_field()
    f.upload(a)
    return f


def test_static_sync_matches_context_sync_two_calls():
    op = _op(48)
    rng = np.random.default_rng(20261203)
    L = op._L
    for _ in range(2):   # two calls in a row: the second reuses the looked-up scratch
        a = rng.standard_normal((6, op.n, op.n))
        ref = _field(op, a)
        got = _field(op, a)
        op._check(L.swm_sync_scalar(op._h, ref._h))
        op._check(L.swm_sync_scalar_static(op._h, got._h))
        op.synchronize()
        r, g = ref.download(), got.download()
        assert np.max(np.abs(g - r)) <= TOL
        assert not np.array_equal(g, a)   # the sync changed the edge nodes


def test_static_sync_at_its_size_limit_and_beyond():
    top = _op(swm._abi.SWM_SYNC_STATIC_MAX_N)
    L = top._L
    a = np.random.default_rng(7).standard_normal((6, top.n, top.n))
    ref, got = _field(top, a), _field(top, a)
    top._check(L.swm_sync_scalar(top._h, ref._h))
    top._check(L.swm_sync_scalar_static(top._h, got._h))
    top.synchronize()
    assert np.max(np.abs(got.download() - ref.download())) <= TOL
    del ref, got, top

    over = _op(swm._abi.SWM_SYNC_STATIC_MAX_N + 1)
    f = over.create_field()
    rc = L.swm_sync_scalar_static(over._h, f._h)
    assert rc == swm._abi.SWM_E_INVALID
    msg = L.swm_last_error(over._h)
    msg = msg.decode() if isinstance(msg, bytes) else ctypes.string_at(msg).decode()
    assert "static scratch limit" in msg
