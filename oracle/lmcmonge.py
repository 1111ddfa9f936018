"""LMC on a Monge patch: metric, Lan integrator, static kernel (float64).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates
* ``lmcmonge/metrics.py:44-60`` (set_inverse_mass, "fixed"),
  ``:155-166`` (velocity_generator: dense Cholesky of
  diag(M⁻¹) − α²·dl_ig·dl_igᵀ), ``:168-186`` (kinetic_energy),
  ``:188-197`` (set_weighted_gradient, normalizing_constant),
  ``:243-255`` (metric_vector_product), ``:267-284`` (lmcmonge_energy);
* ``lmcmonge/integrators.py:63-155`` (lan_integrator.one_step) and
  ``:158-194`` (half_step_omega), including the missing α² in the
  Sherman–Morrison correction at ``:186-189`` (``alpha2_fix=True`` gives
  the algebraically consistent form instead);
* ``lmcmonge/lmc.py:151-236`` (kernel), ``:472-536`` (lmc_proposal),
  ``:539-565`` (flip_velocity).

It also holds the closed-form O(d) velocity factor that the device uses
(``velocity_closed_form``), checked here against the dense Cholesky.
"""
from __future__ import annotations

from dataclasses import dataclass, replace

import numpy as np

from . import proposal as prop


@dataclass
class MongeState:  # integrators.py:26-40 (RiemannianIntegratorState)
    alpha2: float
    position: np.ndarray
    momentum: np.ndarray
    velocity: np.ndarray
    logdensity: np.ndarray
    logdensity_grad_norm: np.ndarray
    dl_ig: np.ndarray
    Hdl_ig: np.ndarray
    ig_Hdl_ig: np.ndarray
    hv_norm: np.ndarray
    determinant_metric: np.ndarray
    volume_adjustment: np.ndarray


@dataclass
class LMCState:  # lmc.py:32-44
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


def init(target, position):
    """lmc.py:101-109."""
    q = np.asarray(position, dtype=np.float64)
    return LMCState(q, target.logdensity(q), target.grad(q), np.zeros(q.shape[0]))


def normalizing_constant(alpha2, inv_mass, g):
    """metrics.py:193-197: L = 1 + α² (M⁻¹∇ℓ)·∇ℓ."""
    return 1.0 + alpha2 * np.sum(inv_mass * g * g, axis=1)


def kinetic_energy(v, alpha2, g_norm, L, mass):
    """metrics.py:168-186."""
    return (
        -0.5 * (np.log(L) + np.sum(np.log(mass)))
        + 0.5 * np.sum(mass * v * v, axis=1)
        + 0.5 * L * alpha2 * np.sum(v * g_norm, axis=1) ** 2
    )


def metric_vector_product(v, alpha2, g, L, mass):
    """metrics.py:243-255 (called with the RAW gradient, lmc.py:202-204)."""
    return v * mass + (alpha2 * L * np.sum(v * g, axis=1))[:, None] * g


def velocity_dense(alpha2, inv_mass, dl_ig, z):
    """metrics.py:155-166: v = chol(diag(M⁻¹) − α² w wᵀ)·z."""
    C, d = dl_ig.shape
    A = np.eye(d)[None] * inv_mass[None, :, None] - alpha2 * dl_ig[:, :, None] * dl_ig[:, None, :]
    Lc = np.linalg.cholesky(A)
    return np.einsum("cij,cj->ci", Lc, z)


def velocity_closed_form(alpha2, inv_mass, dl_ig, z, L):
    """Same L·z as ``velocity_dense`` in O(d), as the device computes it.

    With D = diag(M⁻¹), u = D^{-1/2} w and c = α², the Cholesky factor of
    I − c·uuᵀ is l_jj = sqrt(τ_{j+1}/τ_j), l_ij = −c·u_i·u_j/sqrt(τ_j τ_{j+1})
    (i > j) with τ_j = 1 − cΣ_{k<j} u_k² (the rank-one modification of
    Gill, Golub, Murray & Saunders, 1974).  Because τ_d = 1/L, the suffix
    form τ_j = 1/L + cΣ_{k≥j} u_k² is used (no cancellation).
    """
    c = alpha2
    sd = np.sqrt(inv_mass)[None, :]
    u = dl_ig / sd
    u2 = u * u
    suffix = np.cumsum(u2[:, ::-1], axis=1)[:, ::-1]  # Σ_{k≥j}
    tau = 1.0 / L[:, None] + c * suffix  # τ_j
    tau_next = tau - c * u2  # τ_{j+1}
    r = np.sqrt(tau * tau_next)
    t = u * z / r
    prefix = np.cumsum(t, axis=1) - t  # Σ_{j<i}
    y = np.sqrt(tau_next / tau) * z - c * u * prefix
    return sd * y


def half_step_omega(alpha2, v, J, dl, Hv, L, dl_ig, Hdl_ig, ig_Hdl_ig, eps, alpha2_fix=False):
    """integrators.py:158-194."""
    dot = lambda a, b: np.sum(a * b, axis=1)
    det1 = 1.0 + 0.5 * eps * alpha2 * dot(Hv, dl_ig)
    J = J - np.log(np.abs(det1))
    sL = np.sqrt(L)
    dphi = -dl + alpha2 * Hdl_ig / sL[:, None]
    dphi_ig = -dl_ig + alpha2 * ig_Hdl_ig / sL[:, None]
    v_temp = v - 0.5 * eps * sL[:, None] * (dphi_ig - (alpha2 * dot(dphi, dl_ig))[:, None] * dl_ig)
    corr = 0.5 * eps * dot(v_temp, Hv) / det1
    if alpha2_fix:
        corr = alpha2 * corr
    v_new = v_temp - corr[:, None] * dl_ig
    J = J + np.log(np.abs(1.0 - 0.5 * eps * alpha2 * dot(Hdl_ig, v_new)))
    return v_new, J


def lan_step(target, s: MongeState, eps, inv_mass, mass, alpha2_fix=False):
    """integrators.py:63-155."""
    a2 = s.alpha2
    v, J = half_step_omega(a2, s.velocity, s.volume_adjustment, s.logdensity_grad_norm, s.hv_norm,
                           s.determinant_metric, s.dl_ig, s.Hdl_ig, s.ig_Hdl_ig, eps, alpha2_fix)
    q = s.position + eps * v
    ld, g = target.logdensity(q), target.grad(q)
    L = normalizing_constant(a2, inv_mass, g)
    sL = np.sqrt(L)[:, None]
    g_n = g / sL
    hv_n = target.hvp(q, v) / sL
    dl_ig = inv_mass * g_n
    Hdl_ig = target.hvp(q, dl_ig) / sL
    ig_Hdl_ig = inv_mass * Hdl_ig
    v, J = half_step_omega(a2, v, J, g_n, hv_n, L, dl_ig, Hdl_ig, ig_Hdl_ig, eps, alpha2_fix)
    hv_n = target.hvp(q, v) / sL
    mom = metric_vector_product(v, a2, g, L, mass)
    return MongeState(a2, q, mom, v, ld, g_n, dl_ig, Hdl_ig, ig_Hdl_ig, hv_n, L, J)


def energy(s: MongeState, mass):
    """lmcmonge_energy, metrics.py:267-284."""
    return -s.logdensity + kinetic_energy(s.velocity, s.alpha2, s.logdensity_grad_norm,
                                          s.determinant_metric, mass) - s.volume_adjustment


def kernel(target, state: LMCState, z, u, step_size, inverse_mass_matrix, num_integration_steps,
           alpha2=0.001, *, divergence_threshold=1000.0, alpha2_fix=False, closed_form_velocity=False,
           trajectory=None):
    """lmc.py:151-236 + lmc_proposal :472-536.  z: [C, d] normals, u: [C]."""
    q = state.position
    inv_mass = np.asarray(inverse_mass_matrix, dtype=np.float64)  # "fixed" (metrics.py:48-49)
    mass = 1.0 / inv_mass
    L = normalizing_constant(alpha2, inv_mass, state.logdensity_grad)
    sL = np.sqrt(L)[:, None]
    g_n = state.logdensity_grad / sL
    dl_ig = inv_mass * g_n
    Hdl_ig = target.hvp(q, dl_ig) / sL
    ig_Hdl_ig = inv_mass * Hdl_ig
    if closed_form_velocity:
        v = velocity_closed_form(alpha2, inv_mass, dl_ig, z, L)
    else:
        v = velocity_dense(alpha2, inv_mass, dl_ig, z)
    mom = metric_vector_product(v, alpha2, state.logdensity_grad, L, mass)
    hv_n = target.hvp(q, v) / sL
    s0 = MongeState(alpha2, q, mom, v, state.logdensity, g_n, dl_ig, Hdl_ig, ig_Hdl_ig, hv_n, L,
                    state.volume_adjustment)
    s = s0
    for _ in range(num_integration_steps):
        s = lan_step(target, s, step_size, inv_mass, mass, alpha2_fix)
        if trajectory is not None:
            trajectory.append(s)
    s = replace(s, velocity=-s.velocity, momentum=-s.momentum)  # flip_velocity, lmc.py:539-565
    H0 = energy(s0, mass)
    H1 = energy(s, mass)
    w = prop.energy_diff_weight(H0, H1)
    div = prop.is_divergent(w, divergence_threshold)
    acc, p_acc = prop.static_accept(w, u)
    a = acc[:, None]
    grad_prop = s.logdensity_grad_norm * np.sqrt(s.determinant_metric)[:, None]  # lmc.py:231
    new = LMCState(
        np.where(a, s.position, state.position),
        np.where(acc, s.logdensity, state.logdensity),
        np.where(a, grad_prop, state.logdensity_grad),
        np.where(acc, s.volume_adjustment, state.volume_adjustment),
    )
    return new, LMCInfo(v, p_acc, acc, div, H1, num_integration_steps, s)
