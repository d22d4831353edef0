"""Shared helpers of the GPU parity tests."""
import numpy as np


def rel_l2(a, b, J):
    """J-weighted relative L2 difference (vec_math_mod.f90:50-90 weighting)."""
    num = np.sqrt(np.sum(J * (a - b) ** 2))
    den = np.sqrt(np.sum(J * b ** 2))
    return float(num / den) if den > 0 else float(num)


def fmt7(x):
    return "%.6E" % x
