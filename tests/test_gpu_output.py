"""Lat-lon and paneled output on the GPU.

- The reference's regrid known-answer values (test_regrid_mod.f90, Ah grid,
  N=32, Nlon=4N, Nlat=2N+1; tests/golden/regrid_ah_n32.json) reproduced
  through the C-ABI to 1e-9 relative: maximum errors of the xyz scalar field
  and of the solid rotation field (covariant and contravariant components),
  linear and cubic.
- The regrid of model states against the oracle (FP64, 1e-13 of the field's
  size) and the FP32 pair against FP64.
- The files: FP32 direct-access records of Nlon*Nlat (lat-lon) or
  6*(N+1)^2 (paneled) values, record k at byte (k-1)*count*4."""
import json
import os

import numpy as np
import pytest

import cubedsphere_sbp_swm_gb300 as swm
from cubedsphere_sbp_swm_gb300 import _abi, initial
import oracle

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "regrid_ah_n32.json")))


def _latlon_xyz(nlon, nlat):
    lon = 2.0 * np.pi / nlon * np.arange(nlon)
    lat = -0.5 * np.pi + np.pi / (nlat - 1.0) * np.arange(nlat)
    LAT, LON = np.meshgrid(lat, lon, indexing="ij")
    return LAT, LON, np.cos(LAT) * np.cos(LON), np.cos(LAT) * np.sin(LON), np.sin(LAT)


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['kind']}-{c['components']}-{c['interp']}")
def test_regrid_known_answers_through_the_gpu(case):
    N, nlon, nlat = 32, 128, 65
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, radius=1.0, omega=1.0, precision="fp64"))
    od = oracle.OracleDomain(N, 42, radius=1.0, omega=1.0)
    comps = case["components"] or "covariant"
    rg = swm.LatLonRegrid(op, nlon, nlat, case["interp"], comps)
    LAT, LON, x, y, z = _latlon_xyz(nlon, nlat)
    err = np.zeros(2)
    fa, fb = op.create_field(), op.create_field()
    for k in range(3):
        if case["kind"] == "scalar":
            fa.upload(od.scalar_test_field("xyz", k))
            got = rg.do_regrid(fa)
            err[0] = max(err[0], np.abs(got - (x, y, z)[k]).max())
        else:
            u, v = od.vector_test_field("solid_rotation", k, contravariant=comps == "contravariant")
            fa.upload(u)
            fb.upload(v)
            ug, vg = rg.do_regrid_vec(fa, fb)
            ax = np.eye(3)[k]
            w = np.cross(ax, np.stack([x, y, z], -1))   # solid rotation about axis k
            ut = -np.sin(LON) * w[..., 0] + np.cos(LON) * w[..., 1]
            vt = (-np.sin(LAT) * np.cos(LON) * w[..., 0] - np.sin(LAT) * np.sin(LON) * w[..., 1]
                  + np.cos(LAT) * w[..., 2])
            err[0] = max(err[0], np.abs(ug - ut).max())
            err[1] = max(err[1], np.abs(vg - vt).max())
    ref = np.array(case["values"])
    assert np.allclose(err[:len(ref)], ref, rtol=1e-9, atol=0.0), (err, ref)


@pytest.mark.parametrize("interp,width", [("linear", 2), ("cubic", 4)])
def test_state_regrid_matches_oracle(interp, width):
    N, nlon, nlat = 48, 4 * 48, 2 * 48 + 1
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision="fp64"))
    od = oracle.OracleDomain(N, 42)
    h, u, v, _ = initial.balanced_zonal(N, 2, 16)
    s = op.create_stvec()
    s.upload(h, u, v)
    rg = swm.LatLonRegrid(op, nlon, nlat, interp, "covariant")
    hg, ug, vg = rg.regrid_state(s)
    ho = od.latlon_scalar(h, nlon, nlat, width)
    uo, vo = od.latlon_vector(u, v, nlon, nlat, width, contravariant=False)
    assert np.abs(hg - ho).max() <= 1e-13 * np.abs(ho).max()
    assert np.abs(ug - uo).max() <= 1e-13 * np.abs(uo).max()
    assert np.abs(vg - vo).max() <= 1e-13 * np.abs(uo).max()


def test_fp32_state_regrid_uses_the_pair():
    N = 48
    res = {}
    for prec in ("fp64", "fp32"):
        op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision=prec))
        h, u, v, _ = initial.balanced_zonal(N, 2, 16)
        s = op.create_stvec()
        s.upload(h, u, v)
        res[prec] = swm.LatLonRegrid(op, 4 * N, 2 * N + 1).regrid_state(s)
    # the (hi, lo) pair holds the state to ~2^-48 relative; the north
    # component of a zonal flow is a cancellation of east-component-sized
    # terms, so vector errors are measured against the vector's size
    (h32, u32, v32), (h64, u64, v64) = res["fp32"], res["fp64"]
    vscale = max(np.abs(u64).max(), np.abs(v64).max())
    assert np.abs(h32 - h64).max() <= 1e-12 * np.abs(h64).max()
    assert np.abs(u32 - u64).max() <= 1e-12 * vscale
    assert np.abs(v32 - v64).max() <= 1e-12 * vscale


def test_latlon_and_paneled_files(tmp_path):
    N = 32
    nlon, nlat = 4 * N, 2 * N + 1
    op = swm.OperatorSWM(swm.ModelConfig(N=N, sbp_order=42, precision="fp64"))
    h, u, v, _ = initial.balanced_zonal(N, 2, 16)
    s1, s2 = op.create_stvec(), op.create_stvec()
    s1.upload(h, u, v)
    s2.upload(h + 100.0, 2.0 * u, -v)
    out = swm.LatLonOutputer(op, nlat, nlon)
    names = [str(tmp_path / f) for f in ("h.dat", "u.dat", "v.dat")]
    out.write(s1, *names, rec_num=1)
    out.write(s2, *names, rec_num=2)
    for rec, s in ((0, s1), (1, s2)):
        ref = out.regrid.regrid_state(s)
        for name, r in zip(names, ref):
            data = np.fromfile(name, dtype=np.float32).reshape(2, nlat, nlon)
            assert np.array_equal(data[rec], r.astype(np.float32))
    pan = swm.PaneledOutputer(op)
    pfile = str(tmp_path / "hp.dat")
    pan.write(s2, 0, pfile, rec_num=2)
    data = np.fromfile(pfile, dtype=np.float32).reshape(2, 6, N + 1, N + 1)
    assert np.array_equal(data[1], (h + 100.0).astype(np.float32))
    assert not data[0].any()   # the unwritten first record reads as zeros


def test_output_errors(tmp_path):
    op = swm.OperatorSWM(swm.ModelConfig(N=32, sbp_order=42, precision="fp64"))
    with pytest.raises(swm.SwmError) as e:
        swm.LatLonRegrid(op, 128, 65, "quintic")
    assert e.value.code == _abi.SWM_E_UNSUPPORTED
    with pytest.raises(swm.SwmError) as e:
        swm.LatLonRegrid(op, 128, 65, "cubic", "physical")
    assert e.value.code == _abi.SWM_E_UNSUPPORTED
    s = op.create_stvec()
    out = swm.LatLonOutputer(op, 65, 128)
    with pytest.raises(swm.SwmError) as e:
        out.write(s, str(tmp_path / "h.dat"), None, None, rec_num=0)
    assert e.value.code == _abi.SWM_E_INVALID
    with pytest.raises(swm.SwmError) as e:
        out.write(s, str(tmp_path / "missing_dir" / "h.dat"), None, None, rec_num=1)
    assert e.value.code == _abi.SWM_E_IO
