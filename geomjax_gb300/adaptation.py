"""Host-side adaptation loops driving the device kernels.

Restates the reference's Stan-style warm-up:
* ``dual_averaging`` (``optimizers/dual_averaging.py:53-129``) and its
  step-size wrapper (``adaptation/step_size.py:65-150``);
* ``welford_covariance`` (``adaptation/mass_matrix.py:159-260``) and the
  regularised ``mass_matrix_adaptation`` final step (``:131-154``);
* ``build_schedule`` (``adaptation/window_adaptation.py:360-450``);
* ``window_adaptation`` (``window_adaptation.py:245-357``) and
  ``step_size_adaptation`` (``adaptation/step_size_adaptation.py:100-203``).

The adaptation loops drive the static-length samplers (``rmhmc``, ``lmc``,
``lmcmonge``) and the NUTS samplers (``nutsrmhmc``, ``nutslmc``,
``nutslmcmonge``), each through its own kernel signature.

Batching: the reference adapts one chain (users vmap it).  Here all chains
of a context share one step size (the kernels take a scalar step size): the
dual-averaging statistic is the mean acceptance probability over chains and
the Welford estimator pools every chain's position.  The reference's
``window_adaptation`` passes the adapted inverse mass matrix as the 5th
positional kernel argument (``window_adaptation.py:303-310``), which only
fits the LMC-Monge kernel (``lmcmonge/lmc.py:156``); for ``rmhmc`` / ``lmc``
(whose 5th argument is the metric) only the step size is adapted, as
``step_size_adaptation`` does.
"""
from __future__ import annotations

import math
from typing import NamedTuple

import torch

from .base import AdaptationAlgorithm, AdaptationResults
from .samplers import lmc, lmcmonge, rmhmc


class DualAveragingState(NamedTuple):
    log_step_size: float
    log_step_size_avg: float
    step: int
    avg_error: float
    mu: float


def dual_averaging_init(initial_step_size: float) -> DualAveragingState:
    """dual_averaging.py:87-99: μ = log(10·ε₀)."""
    return DualAveragingState(math.log(initial_step_size), 0.0, 1, 0.0,
                              math.log(10.0 * initial_step_size))


def dual_averaging_update(s: DualAveragingState, gradient: float, t0=10, gamma=0.05,
                          kappa=0.75) -> DualAveragingState:
    """dual_averaging.py:101-123 (``gradient`` = target − acceptance)."""
    reg = s.step + t0
    eta = s.step ** (-kappa)
    avg_error = (1.0 - 1.0 / reg) * s.avg_error + gradient / reg
    log_x = s.mu - (math.sqrt(s.step) / gamma) * avg_error
    log_x_avg = eta * s.log_step_size + (1.0 - eta) * s.log_step_size_avg
    return DualAveragingState(log_x, log_x_avg, s.step + 1, avg_error, s.mu)


class WelfordState(NamedTuple):
    mean: torch.Tensor
    m2: torch.Tensor
    count: int


def welford_init(d, diagonal=True, device="cpu"):
    z = torch.zeros(d, dtype=torch.float64, device=device)
    return WelfordState(z, z.clone() if diagonal else torch.zeros(d, d, dtype=torch.float64,
                                                                  device=device), 0)


def welford_update(s: WelfordState, value: torch.Tensor) -> WelfordState:
    """mass_matrix.py:206-230 (the pooled estimator over chains).

    The reference folds in one sample per call.  A [C, d] batch of chain
    positions is folded in at once by the pairwise combination of two
    Welford states (Chan, Golub and LeVeque 1979): the batch's own mean and
    sum of squared deviations, then n·n_b/(n + n_b)·δδᵀ for the shift
    between the two means.  The result is the row-by-row recursion's up to
    rounding, in a handful of kernels whatever C is."""
    value = value.double()
    if value.ndim == 1:
        value = value[None]
    n_b = value.shape[0]
    if n_b == 0:
        return s
    mean_b = value.mean(0)
    dev = value - mean_b
    m2_b = (dev * dev).sum(0) if s.m2.ndim == 1 else dev.T @ dev
    n = s.count
    tot = n + n_b
    delta = mean_b - s.mean
    mean = s.mean + delta * (n_b / tot)
    w = n * n_b / tot
    m2 = s.m2 + m2_b + (delta * delta * w if s.m2.ndim == 1 else torch.outer(delta, delta) * w)
    return WelfordState(mean, m2, tot)


def welford_covariance(s: WelfordState):
    """mass_matrix.py:232-260: covariance = m2 / (n − 1)."""
    return s.m2 / (s.count - 1), s.count, s.mean


def regularized_inverse_mass(s: WelfordState):
    """mass_matrix.py:131-154 (Stan's shrinkage)."""
    cov, n, mean = welford_covariance(s)
    scaled = (n / (n + 5.0)) * cov
    shrink = 1e-3 * (5.0 / (n + 5.0))
    if scaled.ndim == 1:
        return scaled + shrink
    return scaled + shrink * torch.eye(mean.shape[0], dtype=scaled.dtype, device=scaled.device)


def build_schedule(num_steps: int, initial_buffer_size=75, final_buffer_size=50,
                   first_window_size=25):
    """window_adaptation.py:360-450; list of (stage, is_middle_window_end)."""
    schedule = []
    if num_steps < 20:
        return [(0, False)] * num_steps
    if initial_buffer_size + first_window_size + final_buffer_size > num_steps:
        initial_buffer_size = int(0.15 * num_steps)
        final_buffer_size = int(0.1 * num_steps)
        first_window_size = num_steps - initial_buffer_size - final_buffer_size
    schedule += [(0, False)] * (initial_buffer_size - 1)
    schedule.append((0, False))
    final_buffer_start = num_steps - final_buffer_size
    next_size = first_window_size
    next_start = initial_buffer_size
    while next_start < final_buffer_start:
        cur_start, cur_size = next_start, next_size
        if 3 * cur_size <= final_buffer_start - cur_start:
            next_size = 2 * cur_size
        else:
            cur_size = final_buffer_start - cur_start
        next_start = cur_start + cur_size
        schedule += [(1, False)] * (next_start - 1 - cur_start)
        schedule.append((1, True))
    schedule += [(0, False)] * (num_steps - 1 - final_buffer_start)
    schedule.append((0, False))
    return schedule


def _stepper(algorithm, extra):
    """(step(gen, state, target, step_size, inverse_mass), init, adapts the
    mass) for a static-length sampler (extra: num_integration_steps, alpha2
    for lmcmonge) or a NUTS sampler (extra: max_num_doublings, alpha2 for
    nutslmcmonge), each called with its own kernel signature."""
    from .nuts import nutslmc, nutslmcmonge, nutsrmhmc

    if algorithm is rmhmc or algorithm is lmc or algorithm is lmcmonge:
        kernel = algorithm.build_kernel()
        L = int(extra["num_integration_steps"])
        monge = algorithm is lmcmonge

        def step(gen, state, target, h, inv_mass):
            kw = dict(alpha2=extra.get("alpha2", 0.001), inverse_mass_matrix=inv_mass) if monge \
                else {}
            return kernel(gen, state, target, h, L, **kw)

        return step, algorithm.init, monge
    if algorithm is nutsrmhmc or algorithm is nutslmc:
        kernel = algorithm.build_kernel()
        M = int(extra.get("max_num_doublings", 10))

        def step(gen, state, target, h, inv_mass):
            return kernel(gen, state, target, h, M)

        return step, algorithm.init, False
    if algorithm is nutslmcmonge:
        kernel = algorithm.build_kernel(max_num_doublings=int(extra.get("max_num_doublings", 10)))

        def step(gen, state, target, h, inv_mass):
            return kernel(gen, state, target, h, inv_mass, extra.get("alpha2", 0.001))

        return step, algorithm.init, True
    raise ValueError("algorithm must be one of geomjax_gb300's rmhmc, lmc, lmcmonge, nutsrmhmc, "
                     "nutslmc, nutslmcmonge")


def window_adaptation(algorithm, target, is_mass_matrix_diagonal=True, initial_step_size=1.0,
                      target_acceptance_rate=0.80, progress_bar=False, **extra_parameters):
    """window_adaptation.py:245-357.  ``extra_parameters``: for the static
    samplers ``num_integration_steps``, for NUTS ``max_num_doublings``
    (default 10); ``alpha2`` for the Monge samplers, whose diagonal inverse
    mass matrix is adapted too."""
    kstep, init, adapt_mass = _stepper(algorithm, extra_parameters)
    if adapt_mass and not is_mass_matrix_diagonal:
        raise ValueError("the Monge metric takes a diagonal inverse mass matrix")

    def run(rng_key, position, num_steps: int = 1000):
        gen = rng_key if isinstance(rng_key, torch.Generator) else \
            torch.Generator(device=target.device).manual_seed(int(rng_key))
        state = init(position, target)
        d = target.dim
        da = dual_averaging_init(initial_step_size)
        step_size = initial_step_size
        wf = welford_init(d, True, target.device)
        inv_mass = torch.ones(d, dtype=target.dtype, device=target.device)
        infos = []
        for stage, is_end in build_schedule(num_steps):
            state, info = kstep(gen, state, target, step_size, inv_mass)
            acc = float(info.acceptance_rate.mean().item())
            infos.append(acc)
            if stage == 1 and adapt_mass:
                wf = welford_update(wf, state.position)
            da = dual_averaging_update(da, target_acceptance_rate - acc)
            step_size = math.exp(da.log_step_size)
            if is_end:  # slow_final (window_adaptation.py:174-190)
                if adapt_mass and wf.count > 1:
                    inv_mass = regularized_inverse_mass(wf).to(target.dtype)
                    wf = welford_init(d, True, target.device)
                da = dual_averaging_init(math.exp(da.log_step_size_avg))
                step_size = math.exp(da.log_step_size)
        params = {"step_size": math.exp(da.log_step_size_avg), **extra_parameters}
        if adapt_mass:
            params["inverse_mass_matrix"] = inv_mass
        return AdaptationResults(state, params), infos

    return AdaptationAlgorithm(run)


def step_size_adaptation(algorithm, target, initial_step_size=1.0, target_acceptance_rate=0.80,
                         progress_bar=False, lower_bound=1e-3, **extra_parameters):
    """adaptation/step_size_adaptation.py:100-203 (``extra_parameters`` as
    for ``window_adaptation``; the Monge samplers use the given
    ``inverse_mass_matrix``, ones by default)."""
    kstep, init, _ = _stepper(algorithm, extra_parameters)
    im0 = extra_parameters.get("inverse_mass_matrix")

    def run(rng_key, position, num_steps: int = 1000):
        gen = rng_key if isinstance(rng_key, torch.Generator) else \
            torch.Generator(device=target.device).manual_seed(int(rng_key))
        state = init(position, target)
        da = dual_averaging_init(initial_step_size)
        step_size = initial_step_size
        infos = []
        inv_mass = (torch.ones(target.dim, dtype=target.dtype, device=target.device) if im0 is None
                    else torch.as_tensor(im0).to(device=target.device, dtype=target.dtype))
        for _ in range(num_steps):
            state, info = kstep(gen, state, target, step_size, inv_mass)
            acc = float(info.acceptance_rate.mean().item())
            infos.append(acc)
            da = dual_averaging_update(da, target_acceptance_rate - acc)
            step_size = math.exp(da.log_step_size)
        params = {"step_size": max(math.exp(da.log_step_size_avg), lower_bound),
                  **extra_parameters}
        return AdaptationResults(state, params), infos

    return AdaptationAlgorithm(run)


class GradientStepSizeResult(NamedTuple):
    step_size: float
    mean_acceptance: float
    iterations: int
    history: list  # (step size, mean p_accept, d mean p_accept / dh) per iteration


def gradient_step_size_adaptation(target, positions, num_integration_steps,
                                  initial_step_size=0.05, target_acceptance_rate=0.80,
                                  metric_regulariser=None, num_iterations=40, tol=1e-4, seed=0,
                                  kp=6, kq=6):
    """Step size of generalized-leapfrog RMHMC by a safeguarded Newton method
    on the mean acceptance probability, with its exact derivative from the
    differentiated trajectory (``gj_logreg_gl_transition_jvp``).

    The reference consumes trajectory derivatives the same way in its ChEES
    adaptation, ``jax.jacfwd`` through the integrator
    (``adaptation/chees_adaptation_lmcmonge.py:497-519``), there for the
    trajectory length.  Here the criterion is ⟨min(1, e^{−ΔH})⟩(h) = δ over
    fixed momentum draws (common random numbers), so every iterate solves the
    same equation.  A chain whose transition is not finite counts as
    rejected (p_accept 0, zero derivative), as the reference's accept treats
    a NaN energy.

    Iteration: the step sizes on either side of δ bracket the root; a Newton
    step (derivative negative) is taken when it lands inside the bracket,
    otherwise the bracket is bisected geometrically; before a bracket exists
    h is at most halved or doubled per iteration.  The mean may jump where a
    chain starts to diverge, so the result is within tol of δ, or at such a
    jump with the bracket shrunk to a relative width of 1e-6.  float64
    logistic-regression targets only (d <= 64).
    """
    from . import autodiff as AD

    q0 = torch.as_tensor(positions, dtype=torch.float64).to(target.device).contiguous()
    C, d = q0.shape
    gen = torch.Generator(device="cpu").manual_seed(int(seed))
    z = torch.randn(C, d, generator=gen, dtype=torch.float64).to(target.device)
    lam = 1.0 / target.prior_var if metric_regulariser is None else float(metric_regulariser)
    delta = float(target_acceptance_rate)

    def evaluate(h):
        J = AD.transition_jacobian(target, q0, z, h, lam, num_integration_steps, kp, kq)
        ok = torch.isfinite(J).all(dim=1)
        pa = torch.where(ok, J[:, 0], torch.zeros_like(J[:, 0]))
        dpa = torch.where(ok, J[:, 1], torch.zeros_like(J[:, 1]))
        return float(pa.mean()), float(dpa.mean())

    h = float(initial_step_size)
    lo = hi = None  # step sizes with acceptance above / below the target
    history = []
    it = 0
    pa = float("nan")
    for it in range(1, num_iterations + 1):
        pa, dpa = evaluate(h)
        history.append((h, pa, dpa))
        err = pa - delta
        if abs(err) < tol:
            break
        if err > 0:
            lo = h if lo is None else max(lo, h)
        else:
            hi = h if hi is None else min(hi, h)
        if lo is not None and hi is not None and (hi - lo) < 1e-6 * hi:
            break
        cand = h - err / dpa if dpa < 0 else None
        if lo is not None and hi is not None:
            if cand is None or not (lo < cand < hi):
                cand = math.sqrt(lo * hi)
        else:
            if cand is None or cand <= 0:
                cand = 2.0 * h if err > 0 else 0.5 * h
            cand = min(max(cand, 0.5 * h), 2.0 * h)
        h = cand
    else:
        pa, _ = evaluate(h)
    return GradientStepSizeResult(h, pa, it, history)
