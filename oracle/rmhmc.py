"""RMHMC oracle: Riemannian Gaussian kinetic energy, implicit midpoint with
fixed-point iteration, generalized leapfrog, static kernel (float64).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates
* ``rmhmc/metrics.py:42-127`` (momentum_generator, kinetic_energy,
  inverse_metric_vector_product),
* ``rmhmc/integrators.py:53-89`` (solve_fixed_point_iteration) and
  ``:92-156`` (implicit_midpoint),
* ``rmhmc/rmhmc.py:131-174`` (kernel), ``:376-440`` (rmhmc_proposal),
  ``:443-462`` (flip_momentum), ``mcmc/trajectory.py:121-139``
  (static_integration), ``mcmc/metrics.py:160-166`` (hmc_energy).

The generalized leapfrog is NOT in the reference; it is written from
Girolami & Calderhead (2011), eqs. (16)-(18), and at G = I it reduces to
leapfrog (checked against ``oracle/hmc.py``).

The reference obtains ∂K/∂q with ``jax.grad`` through ``multivariate_normal
.logpdf`` (``rmhmc/integrators.py:112-114``, ``rmhmc/metrics.py:67``).  The
oracle uses the analytic identity
    ∂K/∂q_k = ½ tr(G⁻¹ ∂_k G) − ½ uᵀ ∂_k G u,   u = G⁻¹ p,
which is what that autodiff computes.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import proposal as prop

LOG2PI = np.log(2.0 * np.pi)


# ---------------------------------------------------------------------------
# metric helpers (rmhmc/metrics.py)
# ---------------------------------------------------------------------------
def momentum_from_normals(target, q, z):
    """p = sqrt(G)⊙z (diag) or chol(G)·z (dense); metrics.py:45-58, util.py:83."""
    G = target.metric(q)
    if target.is_diagonal:
        return np.sqrt(G) * z
    L = np.linalg.cholesky(G)
    return np.einsum("cij,cj->ci", L, z)


def inverse_metric_vector_product(target, q, p):
    """v = p / G (diag) or solve(G, p) (dense); metrics.py:120-127."""
    G = target.metric(q)
    if target.is_diagonal:
        return (1.0 / G) * p
    return np.linalg.solve(G, p[..., None])[..., 0]


def kinetic_energy(target, q, p):
    """K = −log N(p; 0, G(q)); metrics.py:60-74 (includes the d/2·log 2π)."""
    G = target.metric(q)
    d = q.shape[1]
    if target.is_diagonal:
        return np.sum(0.5 * p * p / G + 0.5 * np.log(G) + 0.5 * LOG2PI, axis=1)
    L = np.linalg.cholesky(G)
    y = np.linalg.solve(L, p[..., None])[..., 0]
    logdet = 2.0 * np.sum(np.log(np.diagonal(L, axis1=1, axis2=2)), axis=1)
    return 0.5 * np.sum(y * y, axis=1) + 0.5 * logdet + 0.5 * d * LOG2PI


def kinetic_grad(target, q, p):
    """(∂K/∂q, ∂K/∂p) — what ``jax.grad(kinetic_energy, argnums=(0, 1))``
    returns in rmhmc/integrators.py:112-114."""
    G = target.metric(q)
    if target.is_diagonal:
        u = p / G
        dG = target.dmetric(q)  # [C, d, k]
        coef = 0.5 / G - 0.5 * u * u  # [C, d]
        return np.einsum("ca,cak->ck", coef, dG), u
    Ginv = np.linalg.inv(G)
    u = np.einsum("cij,cj->ci", Ginv, p)
    if hasattr(target, "metric_trace_quad"):
        tr, quad = target.metric_trace_quad(q, Ginv, u)
    else:
        dG = target.dmetric(q)  # [C, a, b, k]
        tr = np.einsum("cab,cbak->ck", Ginv, dG)
        quad = np.einsum("ca,cabk,cb->ck", u, dG, u)
    return 0.5 * tr - 0.5 * quad, u


# ---------------------------------------------------------------------------
# fixed point solver (rmhmc/integrators.py:53-89), batched over chains
# ---------------------------------------------------------------------------
@dataclass
class FixedPointInfo:
    success: np.ndarray
    norm: np.ndarray
    iters: np.ndarray


def solve_fixed_point(func, x0, tol=1e-6, divergence_tol=1e10, max_iters=100):
    """x ← func(x) per chain, exactly as the vmapped ``lax.while_loop``:
    one eager evaluation, then iterate while n < max_iters, ‖Δ‖∞ finite,
    < divergence_tol and > tol.  Chains that stop keep their carry.

    ``x0`` is a tuple of [C, ·] arrays; the norm is the ∞-norm over the
    concatenation (``ravel_pytree``)."""

    def norm(a, b):
        return np.max(np.abs(np.concatenate([ai - bi for ai, bi in zip(a, b)], axis=1)), axis=1)

    x = func(x0)
    nrm = norm(x, x0)
    C = nrm.shape[0]
    iters = np.zeros(C, dtype=np.int64)
    with np.errstate(invalid="ignore"):
        active = (iters < max_iters) & np.isfinite(nrm) & (nrm < divergence_tol) & (nrm > tol)
    while active.any():
        xn = func(x)
        nn = norm(xn, x)
        x = tuple(np.where(active[:, None], a, b) for a, b in zip(xn, x))
        nrm = np.where(active, nn, nrm)
        iters = np.where(active, iters + 1, iters)
        with np.errstate(invalid="ignore"):
            active = (iters < max_iters) & np.isfinite(nrm) & (nrm < divergence_tol) & (nrm > tol)
    success = np.isfinite(nrm) & (nrm <= tol)
    return x, FixedPointInfo(success, nrm, iters)


# ---------------------------------------------------------------------------
# integrators
# ---------------------------------------------------------------------------
@dataclass
class IntegratorState:
    position: np.ndarray
    momentum: np.ndarray
    velocity: np.ndarray
    logdensity: np.ndarray
    logdensity_grad: np.ndarray


def implicit_midpoint_step(target, state, h, tol=1e-6, max_iters=100):
    """rmhmc/integrators.py:116-154.  Returns (new_state, FixedPointInfo)."""
    q0, p0 = state.position, state.momentum

    def update(q, p, dldq, initial):
        dTdq, dHdp = kinetic_grad(target, q, p)
        dHdq = dTdq - dldq
        return initial[0] + 0.5 * h * dHdp, initial[1] - 0.5 * h * dHdq

    def step(x):
        q, p = x
        return update(q, p, target.grad(q), (q0, p0))

    (q, p), info = solve_fixed_point(step, (q0, p0), tol=tol, max_iters=max_iters)
    q, p = update(q, p, target.grad(q), (q, p))  # explicit half step (:147-148)
    v = inverse_metric_vector_product(target, q, p)
    return IntegratorState(q, p, v, target.logdensity(q), target.grad(q)), info


def generalized_leapfrog_step(target, state, h, tol=1e-6, max_iters=100):
    """Girolami & Calderhead (2011) eqs. (16)-(18):
        p½ = p − h/2·∂_qH(q, p½)                      (implicit in p)
        q' = q + h/2·[G⁻¹(q) + G⁻¹(q')]·p½            (implicit in q)
        p' = p½ − h/2·∂_qH(q', p½)                    (explicit)
    with ∂_qH = ∂_qK − ∇ℓ.  Both implicit half steps use the same solver
    semantics as the reference (``rmhmc/integrators.py:53-89``)."""
    q0, p0 = state.position, state.momentum
    g0 = state.logdensity_grad

    def p_map(x):
        (p,) = x
        dTdq, _ = kinetic_grad(target, q0, p)
        return (p0 - 0.5 * h * (dTdq - g0),)

    (ph,), info1 = solve_fixed_point(p_map, (p0,), tol=tol, max_iters=max_iters)
    u0 = inverse_metric_vector_product(target, q0, ph)

    def q_map(x):
        (q,) = x
        return (q0 + 0.5 * h * (u0 + inverse_metric_vector_product(target, q, ph)),)

    (q1,), info2 = solve_fixed_point(q_map, (q0,), tol=tol, max_iters=max_iters)
    g1 = target.grad(q1)
    dTdq, _ = kinetic_grad(target, q1, ph)
    p1 = ph - 0.5 * h * (dTdq - g1)
    v = inverse_metric_vector_product(target, q1, p1)
    info = FixedPointInfo(info1.success & info2.success, np.maximum(info1.norm, info2.norm), info1.iters + info2.iters)
    return IntegratorState(q1, p1, v, target.logdensity(q1), g1), info


INTEGRATORS = {
    "implicit_midpoint": implicit_midpoint_step,
    "generalized_leapfrog": generalized_leapfrog_step,
}


# ---------------------------------------------------------------------------
# kernel (rmhmc/rmhmc.py:131-174, 376-462)
# ---------------------------------------------------------------------------
@dataclass
class RMHMCState:
    position: np.ndarray
    logdensity: np.ndarray
    logdensity_grad: np.ndarray


@dataclass
class RMHMCInfo:
    momentum: np.ndarray
    acceptance_rate: np.ndarray
    is_accepted: np.ndarray
    is_divergent: np.ndarray
    energy: np.ndarray
    num_integration_steps: int
    fixed_point_iters: np.ndarray
    fixed_point_success: np.ndarray
    proposal: "IntegratorState" = None  # the flipped end state (rmhmc.py:425-437)


def init(target, position):
    """rmhmc.py:96-98."""
    q = np.asarray(position, dtype=np.float64)
    return RMHMCState(q, target.logdensity(q), target.grad(q))


def hamiltonian(target, s):
    """hmc_energy, mcmc/metrics.py:160-166."""
    return -s.logdensity + kinetic_energy(target, s.position, s.momentum)


def kernel(target, state, z, u, step_size, num_integration_steps, *,
           integrator="implicit_midpoint", tol=1e-6, max_iters=100,
           divergence_threshold=1000.0, trajectory=None):
    """One RMHMC transition for every chain.  ``z``: [C, d] normals for the
    momentum draw, ``u``: [C] uniforms for the accept.  ``trajectory`` (a
    list) receives the IntegratorState after every step when given."""
    step = INTEGRATORS[integrator]
    q = state.position
    p = momentum_from_normals(target, q, z)
    v = inverse_metric_vector_product(target, q, p)
    s0 = IntegratorState(q, p, v, state.logdensity, state.logdensity_grad)
    s = s0
    fp_iters = np.zeros(q.shape[0], dtype=np.int64)
    fp_ok = np.ones(q.shape[0], dtype=bool)
    for _ in range(num_integration_steps):  # trajectory.py:121-139
        s, info = step(target, s, step_size, tol=tol, max_iters=max_iters)
        fp_iters += info.iters
        fp_ok &= info.success
        if trajectory is not None:
            trajectory.append(s)
    s = IntegratorState(s.position, -s.momentum, -s.velocity, s.logdensity, s.logdensity_grad)
    H0 = hamiltonian(target, s0)
    H1 = hamiltonian(target, s)
    w = prop.energy_diff_weight(H0, H1)
    div = prop.is_divergent(w, divergence_threshold)
    acc, p_acc = prop.static_accept(w, u)
    a = acc[:, None]
    new = RMHMCState(
        np.where(a, s.position, state.position),
        np.where(acc, s.logdensity, state.logdensity),
        np.where(a, s.logdensity_grad, state.logdensity_grad),
    )
    info = RMHMCInfo(p, p_acc, acc, div, H1, num_integration_steps, fp_iters, fp_ok, s)
    return new, info
