"""Hyperdiffusion in the CPU oracle: the narrow-stencil SBP Laplacians of
orders 4/2, 6/3 and 2/1 and the biharmonic diffusion operator built on them
(operator_swm_diff_mod.f90:25-46).

The reference holds no golden values for these operators (its Laplacian test
prints errors that reference_results.txt does not record), so the oracle is
pinned by properties that a wrong coefficient, sign or scaling breaks:
- L(1) = 0 to round-off;
- the spherical harmonic Y_2^2 = cos(2 lambda) cos^2(phi) is an eigenfunction
  of the unit-sphere Laplacian with eigenvalue -6 (the reference's own test
  field, test_diffops_mod.f90:180-229): the interior error converges at the
  interior order (4 / 6 / 2), the quadrature-RMS error at about the closure
  order (2 / 3) plus one half (2/1: first-order closure rows, rate 1.5);
- L is symmetric and negative definite in the SBP quadrature inner product
  (relative asymmetry <= 1e-13);
- so the diffusion operator conserves mass (quadrature sum of D h ~ 0) and
  dissipates the quadrature energy (<h, D h> <= 0)."""
import numpy as np
import pytest

import oracle as O

NARROW = (21, 42, 63)


def _ylm22(d):
    g = d.geometry()
    x, y, z = g["rx"], g["ry"], g["rz"]
    lam = np.arctan2(y, x)
    phi = np.arcsin(z / np.sqrt(x * x + y * y + z * z))
    return np.cos(2.0 * lam) * np.cos(phi) ** 2


def _dom(N, narrow, radius=1.0):
    return O.OracleDomain(N, sbp_order=narrow, radius=radius)


@pytest.mark.parametrize("narrow", NARROW)
def test_laplacian_of_a_constant_vanishes(narrow):
    d = _dom(32, narrow, radius=6.371e6)
    L = d.laplace(np.full(d.shape, 5960.0), narrow)
    # a constant of 6e3 m on the Earth: |L| would be ~6e3/(hx a)^2 ~ 1e-4 for
    # an error of one closure coefficient
    assert np.abs(L).max() < 1e-14


@pytest.mark.parametrize("narrow,i_max,r_max,interior_rate,rms_rate",
                         [(42, 4e-5, 3e-3, 14.0, 3.5), (63, 4e-5, 3e-3, 30.0, 6.0),
                          (21, 1e-2, 1.2e-2, 3.8, 2.6)])
def test_spherical_harmonic_eigenvalue_and_convergence(narrow, i_max, r_max, interior_rate, rms_rate):
    errs = []
    for N in (32, 64):
        d = _dom(N, narrow)
        f = _ylm22(d)
        e = np.abs(d.laplace(f, narrow) + 6.0 * f)
        w = 10
        errs.append((e[:, w:-w, w:-w].max(), np.sqrt(d.mass(e * e) / d.mass(np.ones_like(e)))))
    (i32, r32), (i64, r64) = errs
    assert r32 < r_max and i32 < i_max
    assert i32 / i64 > interior_rate
    assert r32 / r64 > rms_rate


@pytest.mark.parametrize("narrow", NARROW)
def test_laplacian_symmetric_negative_definite(narrow):
    rng = np.random.default_rng(7)
    d = _dom(24, narrow)
    f = d.sync_scalar(rng.standard_normal(d.shape))
    g = d.sync_scalar(rng.standard_normal(d.shape))
    Lf, Lg = d.laplace(f, narrow), d.laplace(g, narrow)
    a, b = d.mass(g * Lf), d.mass(f * Lg)
    assert abs(a - b) <= 1e-13 * max(abs(a), abs(b))
    assert d.mass(f * Lf) < 0 and d.mass(g * Lg) < 0


@pytest.mark.parametrize("narrow", NARROW)
def test_biharmonic_is_minus_c4_laplacian_squared(narrow):
    rng = np.random.default_rng(8)
    d = _dom(24, narrow, radius=6.371e6)
    f = d.sync_scalar(rng.standard_normal(d.shape))
    coeff = 0.01
    c = coeff * 6.371e6 * (np.pi / 2 / 24)
    ref = -(c * c) ** 2 * d.laplace(d.laplace(f, narrow), narrow)
    got = d.hordiff_scalar(f, coeff, narrow)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("uv_narrow,h_narrow", [(42, 42), (63, 63), (63, 42), (21, 21)])
def test_diffusion_conserves_mass_and_dissipates(uv_narrow, h_narrow):
    from cubedsphere_sbp_swm_gb300 import initial
    N = 32
    # the h operator conserves mass in the quadrature of its own SBP norm
    d = _dom(N, h_narrow, radius=6.371e6)
    h, u, v, _ = initial.balanced_zonal(N, 2, 16)
    rng = np.random.default_rng(9)
    h = d.sync_scalar(h + 20.0 * rng.standard_normal(d.shape))
    th, tu, tv = d.diffusion_apply(h, u, v, 0.03, 0.01, uv_narrow, h_narrow)
    assert abs(d.mass(th)) <= 1e-12 * d.mass(np.abs(th))
    assert d.mass(h * th) < 0
    assert np.isfinite(tu).all() and np.isfinite(tv).all() and np.abs(tu).max() > 0
    # explicit Euler step = state + dt * tendency
    h1, u1, v1 = d.diffusion_step(h, u, v, 600.0, 0.03, 0.01, uv_narrow, h_narrow)
    for a, b, t in ((h1, h, th), (u1, u, tu), (v1, v, tv)):
        assert np.array_equal(a, b + 600.0 * t)


def test_grid_too_small_for_the_wide_closure_is_rejected():
    d = O.OracleDomain(16, sbp_order=63)   # n = 17 < 2 * 9 closure rows
    f = np.zeros(d.shape)
    out = np.zeros(d.shape)
    assert O.lib().orc_laplace(d._h, 63, O._p(f), O._p(out)) == -1
    assert O.lib().orc_laplace(d._h, 42, O._p(f), O._p(out)) == 0
