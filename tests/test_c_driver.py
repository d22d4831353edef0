"""The C-ABI driven from plain C in the Fortran shim's call order
(tests/c/abi_driver.c; fortran/swm_gpu_shim.f90): the boundary exercised by a
compiled caller, not by ctypes.

CPU: the driver compiles with gcc against include/swm_gpu.h and links
against libswm_gb300.so.  GPU: its RK4 through the abstract interfaces
(apply + assign + update, rk4_mod.f90:20-42) and the fused swm_rk4_step both
match the FP64 oracle, and so do its diagnostics and its hyperdiffusion step
through apply + update (explicit_Eul1_mod.f90:20-30) and the fused step."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from cubedsphere_sbp_swm_gb300 import build as swm_build, initial
from gpu_helpers import rel_l2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "abi_driver.c")
SRC_C = os.path.join(ROOT, "tests", "c", "cgrid_driver.c")


def _compile(tmp_path, src=SRC, name="abi_driver") -> str:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = swm_build.build()
    exe = str(tmp_path / name)
    cmd = [cc, "-O2", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), src,
           "-L", os.path.dirname(lib), "-lswm_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_compiles_and_links(tmp_path):
    assert os.path.exists(_compile(tmp_path))


def test_cgrid_c_driver_compiles_and_links(tmp_path):
    assert os.path.exists(_compile(tmp_path, SRC_C, "cgrid_driver"))


def _run(exe, tmp_path, N, order, prec, dt, nsteps, state):
    np_ = 6 * (N + 1) ** 2
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    np.concatenate([a.ravel() for a in state]).astype(np.float64).tofile(fin)
    r = subprocess.run([exe, str(N), str(order), str(prec), repr(dt), str(nsteps), str(fin), str(fout)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    o = np.fromfile(fout, dtype=np.float64)
    shape = (6, N + 1, N + 1)
    fields = lambda k: [o[(3 * k + c) * np_:(3 * k + c + 1) * np_].reshape(shape) for c in range(3)]
    generic, fused = fields(0), fields(1)
    tail = o[6 * np_:6 * np_ + 9]
    rest = o[6 * np_ + 9:]
    diff_generic = [rest[c * np_:(c + 1) * np_].reshape(shape) for c in range(3)]
    diff_fused = [rest[(3 + c) * np_:(4 + c) * np_].reshape(shape) for c in range(3)]
    return generic, fused, tail[:7], tail[7], tail[8], diff_generic, diff_fused


@pytest.mark.gpu
@pytest.mark.parametrize("order,prec", [(42, 0), (63, 0), (42, 1)], ids=["d42-fp64", "d63-fp64", "d42-fp32"])
def test_c_driver_matches_oracle(tmp_path, order, prec):
    N, dt, nsteps = 48, 300.0, 3
    h, u, v, _ = initial.balanced_zonal(N, 7, 16)
    exe = _compile(tmp_path)
    generic, fused, diag, nrm, dot, dgen, dfus = _run(exe, tmp_path, N, order, prec, dt, nsteps, (h, u, v))
    od = oracle.OracleDomain(N, order)
    J = od.geometry()["J"]
    ref = od.rk4(h, u, v, dt, nsteps)
    tol = nsteps * 1e-12 if prec == 0 else 1e-5
    for g, f, r in zip(generic, fused, ref):
        assert rel_l2(g, r, J) < tol
        assert rel_l2(f, r, J) < tol
    odiag = od.diagnostics(*generic)
    assert np.all(np.abs(diag - odiag) <= (1e-12 if prec == 0 else 1e-7) * np.abs(odiag)), (diag, odiag)
    nref = np.sqrt(sum(np.sum(a * a) for a in generic))
    assert abs(nrm - nref) <= 1e-10 * nref
    dref = sum(np.sum(a * b) for a, b in zip(generic, fused))
    assert abs(dot - dref) <= 1e-10 * abs(dref)
    narrow = 63 if order == 63 else 42
    dref = od.diffusion_step(h, u, v, dt, 0.03, 0.01, narrow, narrow)
    for g, f, r in zip(dgen, dfus, dref):
        assert rel_l2(g, r, J) < (1e-12 if prec == 0 else 1e-6)
        assert rel_l2(f, r, J) < (1e-12 if prec == 0 else 1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("order,prec", [(42, 0), (21, 0), (42, 1)], ids=["c42-fp64", "c21-fp64", "c42-fp32"])
def test_cgrid_c_driver_matches_oracle(tmp_path, order, prec):
    """The C-grid family from plain C: RK4 through the abstract interfaces
    and fused, the curl on a corner-mesh field, the SBP_C mass and the
    drivers' step with the namelist's hyperdiffusion, against the C-grid
    oracle; the refusals of a mixed-order set, of an Ah-grid entry point and
    of an Ah-grid hyperdiffusion name."""
    N, nsteps = 32, 3
    dt = 600.0 * 24 / N
    h, u, v, _ = initial.balanced_zonal_c(N, 4, 12)
    exe = _compile(tmp_path, SRC_C, "cgrid_driver")
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    np.concatenate([a.ravel() for a in (h, u, v)]).astype(np.float64).tofile(fin)
    r = subprocess.run([exe, str(N), str(order), str(prec), repr(dt), str(nsteps), str(fin), str(fout)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    o = np.fromfile(fout, dtype=np.float64)
    shapes = [h.shape, u.shape, v.shape]
    sizes = [a.size for a in (h, u, v)]
    ns = sum(sizes)

    def state(base):
        out, k = [], base
        for sh, n in zip(shapes, sizes):
            out.append(o[k:k + n].reshape(sh))
            k += n
        return out

    generic, fused = state(0), state(ns)
    nq = 6 * (N + 1) ** 2
    curl = o[2 * ns:2 * ns + nq].reshape(6, N + 1, N + 1)
    mass = o[2 * ns + nq]
    od = oracle.OracleCDomain(N, order)
    ref = od.rk4(h, u, v, dt, nsteps)
    tol = nsteps * 1e-12 if prec == 0 else 1e-5

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    for g, f, rr in zip(generic, fused, ref):
        assert rel(g, rr) < tol and rel(f, rr) < tol
    assert rel(curl, od.curl(u, v)) < 1e-12
    assert abs(mass - od.mass(h)) <= 1e-13 * abs(od.mass(h))
    stepped = state(2 * ns + nq + 1)
    ref = od.model_step(h, u, v, dt, nsteps, uv_name="hordiff_c_biharm_curl_div", uv_coeff=0.03, h_coeff=0.03)
    for g, rr in zip(stepped, ref):
        assert rel(g, rr) < tol
