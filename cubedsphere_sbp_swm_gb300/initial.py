"""Seeded synthetic initial states on the cubed sphere (host, FP64, numpy).

These stand in for the reference's analytic test cases (Williamson TS2-type
balanced zonal flow, test_fields_mod.f90:826-859; Galewsky-type barotropic
jet, barotropic_inst_mod.f90:236-284) with seeded perturbations:

* balanced_zonal(N, seed, lmax): u = u0 cos(lat) with u0 ~ U[20, 40] m/s,
  h from the balance relation with area-mean depth 5960 m, plus a random
  spherical-harmonic height perturbation of degrees 1..lmax with amplitude
  spectrum l^-3, rescaled to 10 m area-weighted RMS.  The associated Legendre
  recursion follows random_friction_mod.f90:136-178 (fully normalised P_lm).
* unstable_jet(N, seed): a Gaussian jet in latitude with peak 80 m/s and
  seeded centre/width, its balanced height integrated with 3-point Gauss
  quadrature as barotropic_inst_mod.f90:236-284 does, plus a seeded 120 m
  height bump.

Velocities are returned as covariant components on the unit-sphere basis
(u = V.a1, v = V.a2), the representation the reference stores
(test_fields_mod.f90:283-319).  Arrays have shape (6, N+1, N+1).
"""
from __future__ import annotations

import math
import os

import numpy as np

# panel frames of the six cube faces (ex, ey, inward normal)
_EX = np.array([[-1, 0, 0], [0, 0, -1], [1, 0, 0], [0, 0, 1], [1, 0, 0], [1, 0, 0]], float)
_EY = np.array([[0, 1, 0], [0, 1, 0], [0, 1, 0], [0, 1, 0], [0, 0, 1], [0, 0, -1]], float)
_EN = np.array([[0, 0, 1], [-1, 0, 0], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, -1, 0]], float)

MEAN_DEPTH = 5960.0


def ecs_geometry(N: int, mesh: str = "ah") -> dict:
    """Point positions r (unit sphere), covariant basis a1, a2 and Jacobian J
    of the equiangular cubed sphere (ecs_metric_mod.f90:326-478).  mesh "ah"
    (or "q") is the (N+1) x (N+1) node / corner mesh; the C-grid meshes are
    "p" (N x N cell centres), "u" (x-faces) and "v" (y-faces), with the
    half-cell shifts of mesh_factory_mod.f90:34-41."""
    n = N + 1
    hx = (0.5 * math.pi) / N
    si = 0.5 if mesh in ("p", "v") else 0.0
    sj = 0.5 if mesh in ("p", "u") else 0.0
    al = -0.25 * math.pi + hx * (np.arange(N if si else n) + si)
    be = -0.25 * math.pi + hx * (np.arange(N if sj else n) + sj)
    ta = np.tan(al)[None, :]       # i direction
    tb = np.tan(be)[:, None]       # j direction
    s2 = 1.0 + ta * ta + tb * tb
    sg = np.sqrt(s2)
    p15 = s2 ** 1.5
    one = np.ones_like(s2)
    rp = np.stack([ta * one / sg, tb * one / sg, one / sg], -1)
    a1p = np.stack([(1 + ta * ta) * (1 + tb * tb) / p15, -ta * tb * (1 + ta * ta) / p15,
                    -ta * (1 + ta * ta) * one / p15], -1)
    a2p = np.stack([-ta * tb * (1 + tb * tb) / p15, (1 + ta * ta) * (1 + tb * tb) / p15,
                    -tb * (1 + tb * tb) * one / p15], -1)
    J = (1 + ta * ta) * (1 + tb * tb) / (sg * sg * sg)

    def face(v):
        return (v[None, ..., 0:1] * _EX[:, None, None, :] + v[None, ..., 1:2] * _EY[:, None, None, :]
                - v[None, ..., 2:3] * _EN[:, None, None, :])

    return dict(r=face(rp), a1=face(a1p), a2=face(a2p), J=np.broadcast_to(J, (6,) + J.shape).copy(),
                hx=hx, n=n, N=N)


def _covariant(geo, V):
    return (np.einsum("pjic,pjic->pji", V, geo["a1"]).copy(),
            np.einsum("pjic,pjic->pji", V, geo["a2"]).copy())


def _area_rms(f, J):
    return math.sqrt(float(np.sum(J * f * f) / np.sum(J)))


def _harmonic_block(x, lam, A, B, lmax):
    """sum_m [cos(m lam) S_m + sin(m lam) T_m] over one block of nodes, with
    S_m = sum_l A[l, m] P_lm(x), T_m = sum_l B[l, m] P_lm(x) and the fully
    normalised associated Legendre functions P_lm by the recursion of
    random_friction_mod.f90:136-178 (one order m at a time).  Every node's
    arithmetic is independent of the blocking; the loops work in place."""
    s1 = np.sqrt(1.0 - x * x)
    pmm = np.full_like(x, math.sqrt(0.5))
    f = np.zeros_like(x)
    S, T, p1, p2, t, w = (np.empty_like(x) for _ in range(6))
    for m in range(lmax + 1):
        if m > 0:
            np.multiply(pmm, -math.sqrt((2.0 * m + 1.0) / (2.0 * m)), out=t)
            np.multiply(t, s1, out=pmm)
        S.fill(0.0)
        T.fill(0.0)
        p1[...] = pmm
        for k in range(m, lmax + 1):
            if k == m + 1:
                p2[...] = p1
                np.multiply(p1, math.sqrt(2.0 * m + 3.0), out=t)
                np.multiply(t, x, out=p1)
            elif k > m + 1:
                c1 = math.sqrt((2.0 * k + 1.0) * (2.0 * k - 1.0) / (1.0 * (k + m) * (k - m)))
                c2 = -math.sqrt((2.0 * k + 1.0) * (k - m - 1.0) * (k + m - 1.0)
                                / ((2.0 * k - 3.0) * (k + m) * (k - m)))
                # p_k = (c1 x) p_{k-1} + c2 p_{k-2}; p2 takes p_{k-1}
                np.multiply(x, c1, out=t)
                np.multiply(t, p1, out=t)
                np.multiply(p2, c2, out=p2)
                np.add(t, p2, out=t)
                p2, p1, t = p1, t, p2
            if k >= 1:
                np.multiply(p1, A[k, m], out=w)
                np.add(S, w, out=S)
                if m > 0:
                    np.multiply(p1, B[k, m], out=w)
                    np.add(T, w, out=T)
        if m == 0:
            f += S
        else:
            f += np.cos(m * lam) * S + np.sin(m * lam) * T
    return f


def harmonic_perturbation(geo, seed: int, lmax: int, rms: float = 10.0) -> np.ndarray:
    """Random real spherical-harmonic field, degrees 1..lmax, spectrum l^-3,
    scaled to the given area-weighted RMS.  The coefficients are drawn in
    degree-major order (l = 1..lmax, m = 0..l, two normals each); the sum is
    evaluated over blocks of nodes on the host threads."""
    from concurrent.futures import ThreadPoolExecutor

    rng = np.random.Generator(np.random.PCG64(seed))
    norm = 1.0 / math.sqrt(2.0 * math.pi)
    A = np.zeros((lmax + 1, lmax + 1))
    B = np.zeros((lmax + 1, lmax + 1))
    for l in range(1, lmax + 1):
        amp = float(l) ** -3
        for m in range(0, l + 1):
            a, b = rng.standard_normal(2)
            A[l, m] = amp * a * norm
            B[l, m] = amp * b * norm
    r = geo["r"]
    x = np.ascontiguousarray(r[..., 2]).ravel()    # sin(latitude) about the z axis
    lam = np.arctan2(r[..., 1], r[..., 0]).ravel()
    f = np.empty_like(x)
    blk = 131072

    def run(b0):
        f[b0:b0 + blk] = _harmonic_block(x[b0:b0 + blk], lam[b0:b0 + blk], A, B, lmax)

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(run, range(0, x.size, blk)))
    f = f.reshape(r.shape[:-1])
    return f * (rms / _area_rms(f, geo["J"]))


def balanced_zonal(N: int, seed: int, lmax: int, radius=6.371e6, grav=9.80616, omega=7.292e-5,
                   pert_rms: float = 10.0):
    """Balanced zonal flow u = u0 cos(lat) + seeded height perturbation.
    Returns (h, u, v, info)."""
    geo = ecs_geometry(N)
    rng = np.random.Generator(np.random.PCG64(seed))
    u0 = float(rng.uniform(20.0, 40.0))
    r = geo["r"]
    k = np.array([0.0, 0.0, 1.0])
    V = u0 * np.cross(k, r)                        # u0 cos(lat) e_lambda
    sphi = r[..., 2]
    c = (radius * omega * u0 + 0.5 * u0 * u0) / grav
    H0 = MEAN_DEPTH + c / 3.0                      # area mean of sin^2 = 1/3
    h = H0 - c * sphi * sphi
    if pert_rms > 0.0 and lmax > 0:
        h = h + harmonic_perturbation(geo, seed + 7919, lmax, pert_rms)
    u, v = _covariant(geo, V)
    return h, u, v, dict(u0=u0, H0=H0, seed=seed, lmax=lmax)


def balanced_zonal_c(N: int, seed: int, lmax: int, radius=6.371e6, grav=9.80616, omega=7.292e-5,
                     pert_rms: float = 10.0):
    """balanced_zonal on the C grid: h on the N x N cell centres, covariant u
    on the x-faces and v on the y-faces.  Returns (h, u, v, info)."""
    gp, gu, gv = (ecs_geometry(N, m) for m in ("p", "u", "v"))
    rng = np.random.Generator(np.random.PCG64(seed))
    u0 = float(rng.uniform(20.0, 40.0))
    k = np.array([0.0, 0.0, 1.0])
    sphi = gp["r"][..., 2]
    c = (radius * omega * u0 + 0.5 * u0 * u0) / grav
    H0 = MEAN_DEPTH + c / 3.0
    h = H0 - c * sphi * sphi
    if pert_rms > 0.0 and lmax > 0:
        h = h + harmonic_perturbation(gp, seed + 7919, lmax, pert_rms)
    u = np.einsum("pjic,pjic->pji", u0 * np.cross(k, gu["r"]), gu["a1"]).copy()
    v = np.einsum("pjic,pjic->pji", u0 * np.cross(k, gv["r"]), gv["a2"]).copy()
    return h, u, v, dict(u0=u0, H0=H0, seed=seed, lmax=lmax)


def _jet_u(phi, umax, phic, width):
    return umax * np.exp(-((phi - phic) / width) ** 2)


def unstable_jet(N: int, seed: int, radius=6.371e6, grav=9.80616, omega=7.292e-5,
                 umax: float = 80.0, bump: float = 120.0, nq: int = 4096):
    """Gaussian zonal jet (peak umax) in balance, plus a seeded height bump."""
    geo = ecs_geometry(N)
    rng = np.random.Generator(np.random.PCG64(seed))
    phic = float(rng.uniform(math.pi / 6, math.pi / 3))
    width = float(rng.uniform(0.08, 0.14))
    lam_b = float(rng.uniform(-math.pi, math.pi))
    phi_b = phic + float(rng.uniform(-0.05, 0.05))
    # balance: dh/dphi = -(u^2 tan(phi) + 2 omega a sin(phi) u) / g, Gauss 3-pt
    xq = np.array([-math.sqrt(0.6), 0.0, math.sqrt(0.6)])
    wq = np.array([5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0])
    edges = np.linspace(-0.5 * math.pi, 0.5 * math.pi, nq + 1)
    dphi = edges[1] - edges[0]
    H = np.zeros(nq + 1)
    for jq in range(nq):
        ph = edges[jq] + 0.5 * dphi + 0.5 * dphi * xq
        u = _jet_u(ph, umax, phic, width)
        rhs = -(u * u * np.tan(ph) + 2.0 * omega * radius * np.sin(ph) * u) / grav
        H[jq + 1] = H[jq] + 0.5 * dphi * float(np.sum(wq * rhs))
    r = geo["r"]
    phi = np.arcsin(np.clip(r[..., 2], -1.0, 1.0))
    lam = np.arctan2(r[..., 1], r[..., 0])
    hz = np.interp(phi, edges, H)
    hz = hz - float(np.sum(geo["J"] * hz) / np.sum(geo["J"])) + MEAN_DEPTH
    dl = np.angle(np.exp(1j * (lam - lam_b)))
    h = hz + bump * np.cos(phi) * np.exp(-(dl / (1.0 / 3.0)) ** 2) * np.exp(-((phi - phi_b) / (1.0 / 15.0)) ** 2)
    k = np.array([0.0, 0.0, 1.0])
    kxr = np.cross(k, r)
    cphi = np.maximum(np.linalg.norm(kxr, axis=-1), 1e-14)
    V = (_jet_u(phi, umax, phic, width) / cphi)[..., None] * kxr
    u, v = _covariant(geo, V)
    return h, u, v, dict(phic=phic, width=width, lam_b=lam_b, phi_b=phi_b, seed=seed)


# The benchmark configurations: (N, sbp_order, dt [s], steps, generator args)
CONFIGS = {
    1: dict(N=48, sbp_order=42, dt=900.0, steps=96, seed=1, lmax=16, kind="zonal"),
    2: dict(N=384, sbp_order=42, dt=120.0, steps=7200, seed=2, lmax=64, kind="zonal"),
    4: dict(N=192, sbp_order=42, dt=300.0, steps=240, seed=3, lmax=16, kind="zonal"),
    5: dict(N=1024, sbp_order=63, dt=45.0, steps=9600, seed=5, kind="jet"),
}


def config_state(cfg: int, N: int | None = None, seed: int | None = None):
    """Initial (h, u, v, info) of benchmark configuration cfg (optionally at
    another resolution, for reduced-size parity runs)."""
    c = CONFIGS[cfg]
    N = c["N"] if N is None else N
    seed = c["seed"] if seed is None else seed
    if c["kind"] == "jet":
        return unstable_jet(N, seed)
    return balanced_zonal(N, seed, c["lmax"])
