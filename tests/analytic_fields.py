"""Analytic vector fields of the reference's test_fields_mod.f90 on the unit
sphere, in numpy, evaluated at Cartesian points r (..., 3); shared by the
known-answer and property tests."""
import numpy as np


def cross_polar(r):
    # cross_polar_flow_generator (test_fields_mod.f90), unit sphere
    x, y, z = r[..., 0], r[..., 1], r[..., 2]
    r2 = x * x + y * y + z * z
    cphi, sphi = np.sqrt((x * x + y * y) / r2), z / np.sqrt(r2)
    rho = np.maximum(np.sqrt(x * x + y * y), np.float32(1e-14))
    clam, slam = x / rho, np.where(x * x + y * y == 0.0, 1.0, y / rho)
    u = sphi * (sphi * sphi - 3.0 * cphi * cphi) * slam - 0.5 * cphi
    w = sphi * sphi * clam
    return np.stack([-slam * u - sphi * clam * w, clam * u - sphi * slam * w, cphi * w], -1)


def vsh_curl_free_10(r):
    x, y, z = r[..., 0], r[..., 1], r[..., 2]
    lam = np.arctan2(y, x)
    phi = np.arctan2(z, np.sqrt(x * x + y * y))
    lam = lam + np.pi * (1.0 - np.where(lam >= 0.0, 1.0, -1.0))
    vp = -np.cos(phi)
    return np.stack([-np.sin(phi) * np.cos(lam) * vp, -np.sin(phi) * np.sin(lam) * vp, np.cos(phi) * vp], -1)


def solid_rotation(r, level):
    """solid_rotation_field_generator: the rotation about the coordinate
    axis of the level (x, y, z for levels 0, 1, 2), axis x r."""
    ax = np.eye(3)[level]
    return np.cross(np.broadcast_to(ax, r.shape), r)
