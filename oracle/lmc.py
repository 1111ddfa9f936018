"""Dense-metric LMC (Lan et al. 2015) oracle (float64).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates
* ``lmcmc/metrics.py:75-91`` (velocity_generator, v = L⁻ᵀz),
  ``:93-112`` (kinetic_energy via slogdet), ``:158-179`` (omega_tilde_fn,
  the three einsums over ``jacfwd(metric_fn)``), ``:181-189``
  (grad_logdetmetric = tr(G⁻¹∂_kG)), ``:191-197`` (metric_vector_product),
  ``:209-219`` (lmc_energy);
* ``lmcmc/integrators.py:61-91`` (half_step_fn with LU log-det/solve) and
  ``:93-144`` (one_step);
* ``lmcmc/lmc.py:135-180`` (kernel), ``:411-476`` (lmc_proposal),
  ``:478-500`` (flip_velocity).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import proposal as prop


@dataclass
class LMCState:
    position: np.ndarray
    logdensity: np.ndarray
    logdensity_grad: np.ndarray
    volume_adjustment: np.ndarray


@dataclass
class LMCInfo:
    velocity: np.ndarray
    acceptance_rate: np.ndarray
    is_accepted: np.ndarray
    is_divergent: np.ndarray
    energy: np.ndarray
    num_integration_steps: int
    proposal: object = None  # the flipped end state (position, velocity, ...)


@dataclass
class IntegratorState:  # lmcmc/integrators.py:26-38
    position: np.ndarray
    momentum: np.ndarray
    velocity: np.ndarray
    logdensity: np.ndarray
    logdensity_grad: np.ndarray
    volume_adjustment: np.ndarray


def init(target, position):
    q = np.asarray(position, dtype=np.float64)
    return LMCState(q, target.logdensity(q), target.grad(q), np.zeros(q.shape[0]))


def _dense_metric(target, q):
    G = target.metric(q)
    if target.is_diagonal:
        return G, True
    return 0.5 * (G + np.swapaxes(G, 1, 2)), False


def velocity(target, q, z):
    """metrics.py:75-91: v = L⁻ᵀ z (diag: z/sqrt(G))."""
    G, diag = _dense_metric(target, q)
    if diag:
        return z / np.sqrt(G)
    L = np.linalg.cholesky(G)
    return np.linalg.solve(np.swapaxes(L, 1, 2), z[..., None])[..., 0]


def kinetic_energy(target, q, v):
    """metrics.py:93-112: −½ log det G + ½ vᵀGv."""
    G, diag = _dense_metric(target, q)
    if diag:
        return -0.5 * np.sum(np.log(G), axis=1) + 0.5 * np.sum(G * v * v, axis=1)
    _, logdet = np.linalg.slogdet(G)
    return -0.5 * logdet + 0.5 * np.einsum("ci,cij,cj->c", v, G, v)


def metric_vector_product(target, q, v):
    """metrics.py:191-197 (unsymmetrised G, as the reference)."""
    G = target.metric(q)
    if target.is_diagonal:
        return G * v
    return np.einsum("cij,cj->ci", G, v)


def omega_tilde(target, q, v, h):
    """metrics.py:158-179; returns Ω̃[l, j] per chain.

    For a family whose ∂G is fully symmetric (∂_kG_ij symmetric in i, j, k,
    as Xᵀdiag(Λ'⊙X[:, k])X of logistic regression), the three einsums of
    :174-176 all equal Σ_i v_i ∂_iG, so Ω̃ = G + h/4·Σ_i v_i ∂_iG, formed
    without the d³ tensor (``dmetric_vec``)."""
    G = target.metric(q)
    if getattr(target, "dmetric_fully_symmetric", False):
        return G + 0.25 * h * target.dmetric_vec(q, v)
    dG = target.dmetric(q)
    if target.is_diagonal:
        # dG[c, a, k] = ∂G_a/∂q_k
        p1 = np.einsum("cak,ck->ca", dG, v)
        P1 = np.zeros(dG.shape)
        idx = np.arange(q.shape[1])
        P1[:, idx, idx] = p1
        P2 = dG * v[:, :, None]
        Om = 0.5 * (P1 + P2 - np.swapaxes(P2, 1, 2))
        D = np.zeros(dG.shape)
        D[:, idx, idx] = G
        return D + 0.5 * h * Om
    # dG[c, a, b, k] = ∂G_ab/∂q_k ; einsums of metrics.py:174-176
    p1 = np.einsum("ci,cjli->clj", v, dG)
    p2 = np.einsum("ci,cilj->clj", v, dG)
    p3 = np.einsum("ci,cijl->clj", v, dG)
    return G + 0.5 * h * 0.5 * (p1 + p2 - p3)


def grad_logdetmetric(target, q):
    """metrics.py:181-189: ∂_k log det G = tr(G⁻¹ ∂_k G)."""
    G = target.metric(q)
    if hasattr(target, "metric_trace_quad") and not target.is_diagonal:
        Ginv = np.linalg.inv(G)
        return target.metric_trace_quad(q, Ginv, np.zeros(q.shape))[0]
    dG = target.dmetric(q)
    if target.is_diagonal:
        return np.einsum("ca,cak->ck", 1.0 / G, dG)
    Ginv = np.linalg.inv(G)
    return np.einsum("cab,cbak->ck", Ginv, dG)


def _logabsdet(A):
    """Σ log|diag(U)| of the LU factor = log|det A| (integrators.py:74-76)."""
    return np.linalg.slogdet(A)[1]


def half_step(target, q, v, J, g, h):
    """integrators.py:61-91."""
    Om = omega_tilde(target, q, v, h)
    J = J - _logabsdet(Om)
    dphi = -g + 0.5 * grad_logdetmetric(target, q)
    v_temp = metric_vector_product(target, q, v) - 0.5 * h * dphi
    v_new = np.linalg.solve(Om, v_temp[..., None])[..., 0]
    Om2 = omega_tilde(target, q, v_new, -h)
    J = J + _logabsdet(Om2)
    return v_new, J


def lan_step(target, s: IntegratorState, h):
    """integrators.py:93-144."""
    v, J = half_step(target, s.position, s.velocity, s.volume_adjustment, s.logdensity_grad, h)
    q = s.position + h * v
    ld, g = target.logdensity(q), target.grad(q)
    v, J = half_step(target, q, v, J, g, h)
    mom = metric_vector_product(target, q, v)
    return IntegratorState(q, mom, v, ld, g, J)


def energy(target, s: IntegratorState):
    """lmc_energy, metrics.py:209-219."""
    return -s.logdensity + kinetic_energy(target, s.position, s.velocity) - s.volume_adjustment


def kernel(target, state: LMCState, z, u, step_size, num_integration_steps, *,
           divergence_threshold=1000.0, trajectory=None):
    """lmc.py:135-180 + lmc_proposal."""
    q = state.position
    v = velocity(target, q, z)
    mom = metric_vector_product(target, q, v)
    s0 = IntegratorState(q, mom, v, state.logdensity, state.logdensity_grad, state.volume_adjustment)
    s = s0
    for _ in range(num_integration_steps):
        s = lan_step(target, s, step_size)
        if trajectory is not None:
            trajectory.append(s)
    s = IntegratorState(s.position, -s.momentum, -s.velocity, s.logdensity, s.logdensity_grad,
                        s.volume_adjustment)
    H0 = energy(target, s0)
    H1 = energy(target, s)
    w = prop.energy_diff_weight(H0, H1)
    div = prop.is_divergent(w, divergence_threshold)
    acc, p_acc = prop.static_accept(w, u)
    a = acc[:, None]
    new = LMCState(
        np.where(a, s.position, state.position),
        np.where(acc, s.logdensity, state.logdensity),
        np.where(a, s.logdensity_grad, state.logdensity_grad),
        np.where(acc, s.volume_adjustment, state.volume_adjustment),
    )
    return new, LMCInfo(v, p_acc, acc, div, H1, num_integration_steps, s)
