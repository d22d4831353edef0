"""The host initial-state generator: geometry identical to the oracle's,
and the balanced states are close to steady (small tendencies)."""
import numpy as np

import oracle
from cubedsphere_sbp_swm_gb300 import initial


def test_geometry_matches_oracle():
    d = oracle.OracleDomain(24, 42)
    g = d.geometry()
    b = d.bases()
    geo = initial.ecs_geometry(24)
    assert np.max(np.abs(geo["r"][..., 0] - g["rx"])) < 1e-15
    assert np.max(np.abs(geo["r"][..., 2] - g["rz"])) < 1e-15
    assert np.max(np.abs(geo["a1"] - b["a1"])) < 1e-15
    assert np.max(np.abs(geo["a2"] - b["a2"])) < 1e-15
    assert np.max(np.abs(geo["J"] - g["J"])) < 1e-15


def test_perturbation_rms_and_zero_mean():
    geo = initial.ecs_geometry(32)
    f = initial.harmonic_perturbation(geo, 11, 16, rms=10.0)
    J = geo["J"]
    assert abs(np.sqrt(np.sum(J * f * f) / np.sum(J)) - 10.0) < 1e-9
    assert abs(np.sum(J * f) / np.sum(J)) < 0.5        # degree >= 1: near-zero mean


def test_balanced_state_is_nearly_steady():
    h, u, v, info = initial.balanced_zonal(32, 1, 16, pert_rms=0.0)
    d = oracle.OracleDomain(32, 42)
    th, tu, tv = d.apply(h, u, v)
    # unperturbed balanced flow: the tendency is discretisation error only
    assert np.max(np.abs(th)) < 1e-6 * 5960.0
    assert 20.0 <= info["u0"] <= 40.0


def test_jet_state_is_finite_and_positive():
    h, u, v, info = initial.unstable_jet(32, 5)
    assert np.all(np.isfinite(h)) and np.all(np.isfinite(u)) and np.all(np.isfinite(v))
    assert h.min() > 4000.0
