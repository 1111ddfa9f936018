"""Energy-difference proposal and static Metropolis accept (float64).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``mcmc/proposal.py:87-121`` (``proposal_from_energy_diff``) and
``mcmc/proposal.py:168-185`` (``static_binomial_sampling``), plus the
divergence test of ``rmhmc/rmhmc.py:424`` / ``lmcmonge/lmc.py:520``.
"""
from __future__ import annotations

import numpy as np


def energy_diff_weight(initial_energy, new_energy):
    """w = H0 − H1 with NaN → −∞ (proposal.py:107-108)."""
    with np.errstate(invalid="ignore"):
        w = initial_energy - new_energy
    return np.where(np.isnan(w), -np.inf, w)


def static_accept(w, u):
    """p_accept = min(e^w, 1); accept = u < p_accept (proposal.py:177-178).

    ``jax.random.bernoulli(key, p)`` is ``uniform(key) < p``; the uniform is
    passed in as ``u``.
    """
    with np.errstate(over="ignore"):
        p_accept = np.minimum(np.exp(w), 1.0)
    return u < p_accept, p_accept


def is_divergent(w, threshold=1000.0):
    """rmhmc.py:424: ``-new_proposal.weight > divergence_threshold``."""
    return -w > threshold
