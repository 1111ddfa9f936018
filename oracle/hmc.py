"""Euclidean HMC with velocity Verlet (float64), kept only as the structural
cross-check of ``tests/test_samplers.py:21-57`` (RMHMC with G = I and dense
LMC with G = I must match HMC with ``inverse_mass_matrix = ones``).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``mcmc/integrators.py:47-107`` (velocity_verlet, a1 = 0, b1 = ½)
with a unit diagonal inverse mass matrix, and the static HMC kernel shape of
``mcmc/hmc.py`` (momentum = z, K = ½pᵀp).
"""
from __future__ import annotations

import numpy as np

from . import proposal as prop


def trajectory(target, q, p, h, L):
    g = target.grad(q)
    for _ in range(L):
        p = p + 0.5 * h * g
        q = q + h * p
        g = target.grad(q)
        p = p + 0.5 * h * g
    return q, p


def kernel(target, q, z, u, h, L):
    """Returns (new_position, accepted)."""
    ld0 = target.logdensity(q)
    q1, p1 = trajectory(target, q, z, h, L)
    H0 = -ld0 + 0.5 * np.sum(z * z, axis=1)
    H1 = -target.logdensity(q1) + 0.5 * np.sum(p1 * p1, axis=1)
    w = prop.energy_diff_weight(H0, H1)
    acc, _ = prop.static_accept(w, u)
    return np.where(acc[:, None], q1, q), acc
