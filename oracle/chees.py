"""ChEES adaptation of the step size and the trajectory length (float64).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``adaptation/chees_adaptation_riemanian.py``:

* ``compute_parameters`` (``:104-219``): dual averaging of the step size on
  the harmonic-mean acceptance (``:145-160``), and one optimiser step on the
  log trajectory length along the ChEES gradient (``:162-206``), each
  followed by the moving averages of ``:156-160`` / ``:203-206``;
* ``init`` (``:221-231``), ``run`` / ``one_step`` (``:333-450``) with the
  quasi-random Halton jitter (``:362-366``, ``:468-471``) and
  ``integration_steps_fn`` (``:368-372``);
* the ``lmcmonge`` variant's α² gradient (``chees_adaptation_lmcmonge.py:
  219-256``), as a weighted statistic of a supplied tangent ∂q_L/∂α².

The optimiser the reference passes in (``optax.adam``) is restated from the
published Adam update (Kingma and Ba, 2015) with optax's conventions: bias
correction by the incremented count, ``eps`` added outside the square root,
the update scaled by −learning_rate.

Randomness: per transition the caller passes the normals and uniforms of
every chain (``z``, ``u``) instead of the JAX keys of ``:427``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

OPTIMAL_TARGET_ACCEPTANCE_RATE = 0.651


# -- dual averaging (optimizers/dual_averaging.py:87-123) -------------------
@dataclass
class DualAveragingState:
    log_x: float
    log_x_avg: float
    step: int
    avg_error: float
    mu: float


def da_init(x):
    return DualAveragingState(math.log(x), 0.0, 1, 0.0, math.log(10.0 * x))


def da_update(s, gradient, t0=10, gamma=0.05, kappa=0.75):
    reg = s.step + t0
    eta = s.step ** (-kappa)
    avg_error = (1.0 - 1.0 / reg) * s.avg_error + gradient / reg
    log_x = s.mu - (math.sqrt(s.step) / gamma) * avg_error
    log_x_avg = eta * s.log_x + (1.0 - eta) * s.log_x_avg
    return DualAveragingState(log_x, log_x_avg, s.step + 1, avg_error, s.mu)


# -- Adam with optax's conventions ----------------------------------------
@dataclass
class AdamState:
    count: int
    mu: float
    nu: float


def adam_init(params):
    return AdamState(0, 0.0 * params, 0.0 * params)


def adam_update(g, s, learning_rate, b1=0.9, b2=0.999, eps=1e-8, eps_root=0.0):
    mu = (1.0 - b1) * g + b1 * s.mu
    nu = (1.0 - b2) * g * g + b2 * s.nu
    count = s.count + 1
    mu_hat = mu / (1.0 - b1 ** count)
    nu_hat = nu / (1.0 - b2 ** count)
    lr = learning_rate(s.count) if callable(learning_rate) else learning_rate
    return -lr * mu_hat / (math.sqrt(nu_hat + eps_root) + eps), AdamState(count, mu, nu)


# -- Halton jitter (chees_adaptation_riemanian.py:468-471) ------------------
def halton_sequence(i, max_bits=10):
    return sum(((i + 1) // (2 ** b)) % 2 * (0.5 / 2 ** b) for b in range(int(max_bits)))


# -- cross-chain statistics (chees_adaptation_riemanian.py:145-190) ---------
def statistics(P, V, I, acc, div, D=None):
    """(harmonic mean acceptance, Σ a g / Σ a, Σ a g_α / Σ a) over the
    non-divergent chains, before the jitter × trajectory-length factor."""
    P, V, I = (np.asarray(x, dtype=np.float64) for x in (P, V, I))
    acc = np.asarray(acc, dtype=np.float64)
    keep = ~np.asarray(div, dtype=bool)
    with np.errstate(divide="ignore", invalid="ignore"):
        harmonic = 1.0 / np.mean((1.0 / acc)[keep]) if keep.any() else np.nan
        Pc = P - np.nanmean(P, axis=0)
        Ic = I - np.nanmean(I, axis=0)
        sq = np.sum(Pc * Pc, axis=1) - np.sum(Ic * Ic, axis=1)
        g = sq * np.sum(Pc * V, axis=1)
        wsum = np.sum(acc[keep])
        grad = np.sum((acc * g)[keep]) / wsum
        grad_a = 0.0
        if D is not None:
            ga = sq * np.sum(Pc * np.asarray(D, dtype=np.float64), axis=1)
            grad_a = np.sum((acc * ga)[keep]) / wsum
    return float(harmonic), float(grad), float(grad_a)


@dataclass
class ChEESState:
    step_size: float
    log_step_size_moving_average: float
    trajectory_length: float
    log_trajectory_length_moving_average: float
    da_state: DualAveragingState
    optim_state: AdamState
    random_generator_arg: int
    step: int
    alpha2: float = 1.0
    log_alpha2_moving_average: float = 0.0
    optim_state_alpha2: AdamState = None


def init(random_generator_arg, step_size, alpha2=1.0):
    """chees_adaptation_riemanian.py:221-231 (+ chees_adaptation_lmcmonge.py:
    272-284, whose optimiser state for α² starts from 1.0)."""
    return ChEESState(step_size, 0.0, step_size, 0.0, da_init(step_size), adam_init(step_size),
                      random_generator_arg, 1, alpha2, 0.0, adam_init(1.0))


def compute_parameters(s, harmonic, grad_raw, jitter, learning_rate,
                       target_acceptance_rate=OPTIMAL_TARGET_ACCEPTANCE_RATE, decay_rate=0.5,
                       grad_alpha_raw=None):
    """chees_adaptation_riemanian.py:104-219 given the statistics of
    ``statistics``; ``jitter`` = jitter_generator(random_generator_arg).
    With ``grad_alpha_raw`` also the α² step of chees_adaptation_lmcmonge.py:
    219-256 (its gradient before the jitter × trajectory-length factor)."""
    da_ = da_update(s.da_state, target_acceptance_rate - harmonic)
    step_size_ = math.exp(da_.log_x)
    if math.isfinite(step_size_):
        new_step_size, new_da, new_log_step = step_size_, da_, da_.log_x
    else:
        new_step_size, new_da, new_log_step = s.step_size, s.da_state, s.da_state.log_x
    w = s.step ** (-decay_rate)
    new_log_step_ma = (1.0 - w) * s.log_step_size_moving_average + w * new_log_step
    grad = jitter * s.trajectory_length * grad_raw
    log_T = math.log(s.trajectory_length)
    upd, opt_ = adam_update(grad, s.optim_state, learning_rate)
    log_T_ = log_T + upd
    if math.isfinite(log_T_):
        new_log_T, new_opt = log_T_, opt_
    else:
        new_log_T, new_opt = log_T, s.optim_state
    new_log_T_ma = (1.0 - w) * s.log_trajectory_length_moving_average + w * new_log_T
    alpha2, log_a2_ma, opt_a = s.alpha2, s.log_alpha2_moving_average, s.optim_state_alpha2
    if grad_alpha_raw is not None:
        log_a2 = math.log(s.alpha2)
        upd_a, opt_a_ = adam_update(jitter * s.trajectory_length * grad_alpha_raw,
                                    s.optim_state_alpha2, learning_rate)
        if math.isfinite(log_a2 + upd_a):
            new_log_a2, opt_a = log_a2 + upd_a, opt_a_
        else:
            new_log_a2 = log_a2
        log_a2_ma = (1.0 - w) * s.log_alpha2_moving_average + w * new_log_a2
        alpha2 = math.exp(log_a2_ma)
    return ChEESState(new_step_size, new_log_step_ma, math.exp(new_log_T_ma), new_log_T_ma,
                      new_da, new_opt, s.random_generator_arg + 1, s.step + 1, alpha2, log_a2_ma,
                      opt_a)


def run(transition, positions, step_size, learning_rate, num_steps, *, max_sampling_steps=1000,
        jitter_amount=1.0, target_acceptance_rate=OPTIMAL_TARGET_ACCEPTANCE_RATE, decay_rate=0.5):
    """``run`` with the Halton jitter (``:396-450``).  ``transition(i, state,
    step_size, L)`` performs step i's transition of every chain and returns
    (new_state, info) with ``info.proposal`` and the positions in
    ``state.position``.  Returns the final chain state, the adaptation state,
    the history of adaptation states and the number of integration steps of
    every transition."""
    max_bits = math.ceil(math.log2(num_steps + max_sampling_steps))

    def jitter_gn(i):
        return halton_sequence(i, max_bits) * jitter_amount + (1.0 - jitter_amount)

    s = init(0, step_size)
    state = positions
    hist, lengths = [], []
    for i in range(num_steps):
        L = int(math.ceil(jitter_gn(s.random_generator_arg) * s.trajectory_length / s.step_size))
        new_state, info = transition(i, state, s.step_size, L)
        harmonic, grad_raw, _ = statistics(info.proposal.position, info.proposal.velocity,
                                           state.position, info.acceptance_rate,
                                           info.is_divergent)
        s = compute_parameters(s, harmonic, grad_raw, jitter_gn(s.random_generator_arg),
                               learning_rate, target_acceptance_rate, decay_rate)
        hist.append(replace(s))
        lengths.append(L)
        state = new_state
    return state, s, hist, lengths


def final_parameters(s):
    """``:452-466``: step size and the adjusted trajectory length T/h from
    the moving averages."""
    return (math.exp(s.log_step_size_moving_average),
            math.exp(s.log_trajectory_length_moving_average - s.log_step_size_moving_average))
