"""Host <-> device transfers of states and scalar fields through the C-ABI.

Page-locked host arrays are read and written in place by the pack kernels;
pageable arrays go through a contiguous staging copy; the asynchronous
transfers (swm_state_upload_async / _download_async) go through device
staging buffers on the copy engines.  All routes must give identical device
states.  FP64 round trips are exact; the FP32 (hi, lo) pair
reproduces an FP64 value x to |x - (hi + lo)| <= 2^-47 |x|
(hi = fl32(x) loses at most 2^-24 |x|, lo = fl32(x - hi) keeps all but
2^-24 of that, and the FP64 sum adds at most 2^-53 |x|)."""
import numpy as np
import pytest
import torch

import cubedsphere_sbp_swm_gb300 as swm

pytestmark = pytest.mark.gpu

N = 48


def _pinned_views(shape, count, offset=0, extra=0):
    """count page-locked arrays of `shape`, each starting `offset` doubles
    into its own page-locked allocation of size(shape) + offset + extra."""
    size = int(np.prod(shape))
    bufs = [torch.empty(size + offset + extra, dtype=torch.float64, pin_memory=True)
            for _ in range(count)]
    return bufs, [b.numpy()[offset:offset + size].reshape(shape) for b in bufs]


def _rand(rng, shape):
    return [rng.standard_normal(shape) * 10.0 ** k for k in range(3)]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_page_locked_and_pageable_routes_agree(prec):
    rng = np.random.default_rng(11)
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision=prec))
    sh = op.shape
    x = _rand(rng, sh)
    keep_in, pin_in = _pinned_views(sh, 3, offset=5, extra=37)
    for p, a in zip(pin_in, x):
        p[...] = a
    s_pg, s_pin = op.create_stvec(), op.create_stvec()
    s_pg.upload(*x)
    s_pin.upload(*pin_in)   # read in place over the host link

    out_pg = s_pg.download()
    keep_out, pin_out = _pinned_views(sh, 3)
    s_pin.download(out=tuple(pin_out))
    for a, b, xx in zip(out_pg, pin_out, x):
        assert np.array_equal(a, b)
        if prec == "fp64":
            assert np.array_equal(a, xx)
        else:
            assert np.max(np.abs(a - xx) / np.maximum(np.abs(xx), 1e-300)) <= 2.0 ** -47

    # cross routes: page-locked state into pageable output and back
    out_x = s_pin.download()
    s_pg.download(out=tuple(pin_out))
    for a, b in zip(out_x, pin_out):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_stepped_states_identical_across_routes(prec):
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision=prec))
    from cubedsphere_sbp_swm_gb300 import initial
    h, u, v, _ = initial.balanced_zonal(N, 2, 16)
    keep, pin = _pinned_views(op.shape, 3)
    for p, a in zip(pin, (h, u, v)):
        p[...] = a
    s1, s2 = op.create_stvec(), op.create_stvec()
    s1.upload(h, u, v)
    s2.upload(*pin)
    ts = swm.RK4()
    ts.step(s1, op, 600.0, 3)
    ts.step(s2, op, 600.0, 3)
    for a, b in zip(s1.download(), s2.download()):
        assert np.array_equal(a, b)


def test_scalar_field_routes_agree():
    rng = np.random.default_rng(12)
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision="fp64"))
    a = rng.standard_normal(op.shape)
    keep, pin = _pinned_views(op.shape, 1, offset=3)
    pin[0][...] = a
    f1, f2 = op.create_field(), op.create_field()
    f1.upload(a)
    f2.upload(pin[0])
    assert np.array_equal(f1.download(), a)
    assert np.array_equal(f2.download(), a)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("pinned", [True, False])
def test_async_transfers_match_the_synchronous_route(prec, pinned):
    """upload_async -> steps -> download_async gives the bytes of upload ->
    steps -> download, from page-locked and from pageable arrays."""
    from cubedsphere_sbp_swm_gb300 import initial
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision=prec))
    h, u, v, _ = initial.balanced_zonal(N, 3, 16)
    if pinned:
        keep_in, src = _pinned_views(op.shape, 3)
        keep_out, dst = _pinned_views(op.shape, 3)
    else:
        src = [np.empty(op.shape) for _ in range(3)]
        dst = [np.empty(op.shape) for _ in range(3)]
    for p, a in zip(src, (h, u, v)):
        p[...] = a
    s_sync, s_async = op.create_stvec(), op.create_stvec()
    s_sync.upload(h, u, v)
    s_async.upload_async(*src)
    ts = swm.RK4()
    ts.step(s_sync, op, 600.0, 2)
    ts.step(s_async, op, 600.0, 2)
    s_async.download_async(tuple(dst))
    op.synchronize()
    for a, b in zip(s_sync.download(), dst):
        assert np.array_equal(a, b)


def test_async_pipeline_of_two_states():
    """The pipelined loop the bench's end-to-end figure runs: two states take
    turns; each step uploads its input asynchronously, steps and downloads
    asynchronously, with the next step queued before the last download has
    landed.  Every output equals the synchronous route's, and a state changed
    right after download_async does not change what the download returns."""
    from cubedsphere_sbp_swm_gb300 import initial
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision="fp32"))
    inputs = [initial.balanced_zonal(N, seed, 16)[:3] for seed in (4, 5, 6, 7, 8)]
    expect = []
    ref = op.create_stvec()
    ts = swm.RK4()
    for x in inputs:
        ref.upload(*x)
        ts.step(ref, op, 600.0, 1)
        expect.append(ref.download())
    states = [op.create_stvec(), op.create_stvec()]
    keeps, outs = [], []
    for k, x in enumerate(inputs):
        ki, si = _pinned_views(op.shape, 3)     # every step its own input arrays
        ko, o = _pinned_views(op.shape, 3)
        keeps += [ki, ko]
        outs.append(o)
        for p, a in zip(si, x):
            p[...] = a
        st = states[k % 2]
        st.upload_async(*si)
        ts.step(st, op, 600.0, 1)
        st.download_async(tuple(o))
        st.assign_s1(-1.0)          # changed right after; the download keeps the stepped state
    op.synchronize()
    for e, o in zip(expect, outs):
        for a, b in zip(e, o):
            assert np.array_equal(a, b)


def test_async_transfers_reject_temporaries():
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision="fp64"))
    s = op.create_stvec()
    bad = np.zeros(op.shape, dtype=np.float32)
    good = np.zeros(op.shape)
    with pytest.raises(ValueError):
        s.upload_async(bad, good, good)
    with pytest.raises(ValueError):
        s.download_async((good, good, good[:, ::-1]))
