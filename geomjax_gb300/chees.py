"""ChEES adaptation of the step size and the trajectory length, and the
dynamic (jittered-length) kernels it drives.

Mirrors ``adaptation/chees_adaptation_riemanian.py`` (``chees_adaptation``,
dynamics ``"rmhmc"`` or ``"lmc"``) and ``adaptation/chees_adaptation_lmcmonge.py``
(``lmcmonge_chees_adaptation``), with the dynamic kernels of
``rmhmc/rmhmc.py:179-244``, ``lmcmc/lmc.py:185-252`` and
``lmcmonge/lmc.py:239-309``.

Per warm-up step (``:421-450``): every chain takes one transition with
L = ⌈jitter(i) · T / h⌉ integration steps; the device reduces the proposals
to three numbers (``gj_chees_statistics``: harmonic-mean acceptance, the
ChEES trajectory gradient, the α² gradient); the host then updates the
step size by dual averaging toward the target acceptance and log T by one
optimiser step, each smoothed by a moving average (``:104-219``).  One
three-double device→host read per step is the only synchronisation.

Randomness: ``rng_key`` seeds a ``torch.Generator`` that draws every step's
normals and uniforms on the device (or pass ``draws=[Draws, ...]`` per step).
``jitter_generator``, when given, is called with an integer counter that
starts at 0 and advances by one per transition (the reference threads a JAX
key through ``jax.random.split``); without it the quasi-random Halton
sequence of ``:468-471`` is used.

The reference's LMC-Monge variant cannot run as written: its dynamic kernel
builds ``LMCState`` with an extra ``alpha2`` field and calls the base kernel
without ``alpha2`` (``lmcmonge/lmc.py:281-287``).  ``lmcmonge_chees_adaptation``
implements the evident intent: the adaptation state's α² (the given
``alpha2`` at first) is passed to every transition.  With ``update_alpha``
the α² gradient of ``chees_adaptation_lmcmonge.py:219-256`` uses
∂q_L/∂α² from ``gj_lmcmonge_alpha2_jvp`` (forward mode on the device, where
the reference takes ``jax.jacfwd`` at ``:507``), and α² follows its own
optimiser step and moving average.
"""
from __future__ import annotations

import ctypes
import math
from typing import Any, Callable, NamedTuple, Optional

import torch

from . import _lib as L
from .adaptation import DualAveragingState, dual_averaging_init, dual_averaging_update
from .base import AdaptationAlgorithm, AdaptationResults, Draws, LMCState, RMHMCState
from .autodiff import lmcmonge_alpha2_tangent
from .samplers import Kernel, lmc, lmcmonge, rmhmc
from .targets import PRECISIONS

# optimal tuning for HMC (chees_adaptation_riemanian.py:21)
OPTIMAL_TARGET_ACCEPTANCE_RATE = 0.651


# ---------------------------------------------------------------------------
# optimiser (the reference passes optax.adam)
# ---------------------------------------------------------------------------
class AdamState(NamedTuple):
    count: int
    mu: float
    nu: float


class GradientTransformation(NamedTuple):
    """``optax.GradientTransformation``: init(params) → state,
    update(grad, state, params) → (updates, state)."""

    init: Callable
    update: Callable


def adam(learning_rate, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8,
         eps_root: float = 0.0) -> GradientTransformation:
    """Adam (Kingma and Ba, 2015) on a scalar parameter with optax's
    conventions: moments m ← b1·m + (1−b1)·g, v ← b2·v + (1−b2)·g²; bias
    correction by the incremented count; update
    −lr · m̂ / (√(v̂ + eps_root) + eps).  ``learning_rate`` is a float or a
    function of the step count (an optax schedule)."""

    def init(params):
        return AdamState(0, 0.0, 0.0)

    def update(g, s: AdamState, params=None):
        mu = (1.0 - b1) * g + b1 * s.mu
        nu = (1.0 - b2) * g * g + b2 * s.nu
        count = s.count + 1
        mu_hat = mu / (1.0 - b1 ** count)
        nu_hat = nu / (1.0 - b2 ** count)
        lr = learning_rate(s.count) if callable(learning_rate) else learning_rate
        return -lr * mu_hat / (math.sqrt(nu_hat + eps_root) + eps), AdamState(count, mu, nu)

    return GradientTransformation(init, update)


def _exp(x: float) -> float:
    """exp that overflows to inf (and keeps NaN) instead of raising."""
    if math.isnan(x):
        return math.nan
    return math.exp(x) if x < 709.0 else math.inf


def halton_sequence(i: int, max_bits: int = 10) -> float:
    """Base-2 radical inverse of i + 1 over ``max_bits`` bits
    (chees_adaptation_riemanian.py:468-471)."""
    n = int(i) + 1
    return sum(((n >> b) & 1) * (0.5 / (1 << b)) for b in range(int(max_bits)))


# ---------------------------------------------------------------------------
# adaptation state and update
# ---------------------------------------------------------------------------
class ChEESAdaptationState(NamedTuple):
    """``chees_adaptation_riemanian.py:23-53`` (+ the α² fields of
    ``chees_adaptation_lmcmonge.py``)."""

    step_size: float
    log_step_size_moving_average: float
    trajectory_length: float
    log_trajectory_length_moving_average: float
    da_state: DualAveragingState
    optim_state: Any
    random_generator_arg: int
    step: int
    alpha2: float = 1.0
    log_alpha2_moving_average: float = 0.0
    optim_state_alpha2: Any = None


class ChEESStatistics(NamedTuple):
    harmonic_mean_acceptance: float
    trajectory_gradient: float  # before the jitter × trajectory-length factor
    alpha2_gradient: float


def chees_init(random_generator_arg: int, step_size: float, optim: GradientTransformation,
               alpha2: float = 1.0) -> ChEESAdaptationState:
    """``chees_adaptation_riemanian.py:221-231``: T starts at the step size."""
    return ChEESAdaptationState(step_size, 0.0, step_size, 0.0, dual_averaging_init(step_size),
                                optim.init(step_size), random_generator_arg, 1, alpha2, 0.0,
                                optim.init(1.0))


def chees_update(s: ChEESAdaptationState, stats: ChEESStatistics, jitter: float,
                 optim: GradientTransformation, next_random_arg_fn: Callable,
                 target_acceptance_rate: float = OPTIMAL_TARGET_ACCEPTANCE_RATE,
                 decay_rate: float = 0.5, update_alpha: bool = False) -> ChEESAdaptationState:
    """``compute_parameters`` (``chees_adaptation_riemanian.py:104-219``,
    with ``update_alpha`` the α² step of ``chees_adaptation_lmcmonge.py:
    219-256``) given the device statistics; ``jitter`` is the jitter of this
    step's ``random_generator_arg``."""
    da_ = dual_averaging_update(s.da_state, target_acceptance_rate - stats.harmonic_mean_acceptance)
    step_size_ = _exp(da_.log_step_size)
    if math.isfinite(step_size_):
        new_step_size, new_da, new_log_step = step_size_, da_, da_.log_step_size
    else:
        new_step_size, new_da, new_log_step = s.step_size, s.da_state, s.da_state.log_step_size
    w = s.step ** (-decay_rate)
    new_log_step_ma = (1.0 - w) * s.log_step_size_moving_average + w * new_log_step

    grad = jitter * s.trajectory_length * stats.trajectory_gradient
    log_T = math.log(s.trajectory_length)
    upd, opt_ = optim.update(grad, s.optim_state, log_T)
    log_T_ = log_T + upd
    if math.isfinite(log_T_):
        new_log_T, new_opt = log_T_, opt_
    else:
        new_log_T, new_opt = log_T, s.optim_state
    new_log_T_ma = (1.0 - w) * s.log_trajectory_length_moving_average + w * new_log_T

    alpha2, log_a2_ma, opt_a = s.alpha2, s.log_alpha2_moving_average, s.optim_state_alpha2
    if update_alpha:
        grad_a = jitter * s.trajectory_length * stats.alpha2_gradient
        log_a2 = math.log(s.alpha2)
        upd_a, opt_a_ = optim.update(grad_a, s.optim_state_alpha2, log_a2)
        log_a2_ = log_a2 + upd_a
        if math.isfinite(log_a2_):
            new_log_a2 = log_a2_
            opt_a = opt_a_
        else:
            new_log_a2 = log_a2
        log_a2_ma = (1.0 - w) * s.log_alpha2_moving_average + w * new_log_a2
        alpha2 = _exp(log_a2_ma)
    return ChEESAdaptationState(new_step_size, new_log_step_ma, _exp(new_log_T_ma),
                                new_log_T_ma, new_da, new_opt,
                                next_random_arg_fn(s.random_generator_arg), s.step + 1,
                                alpha2, log_a2_ma, opt_a)


def chees_statistics(proposal_position: torch.Tensor, proposal_velocity: torch.Tensor,
                     initial_position: torch.Tensor, acceptance_rate: torch.Tensor,
                     is_divergent: Optional[torch.Tensor] = None,
                     alpha2_tangent: Optional[torch.Tensor] = None,
                     workspace: Optional[torch.Tensor] = None) -> ChEESStatistics:
    """The cross-chain reductions of ``compute_parameters`` on the device
    (``gj_chees_statistics``); one device→host read of three doubles."""
    P = proposal_position.contiguous()
    C, d = P.shape
    if P.dtype == torch.float64:
        prec = PRECISIONS["fp64"]
    elif P.dtype == torch.float32:
        prec = PRECISIONS["mixed"]
    else:
        raise ValueError("proposals must be float32 or float64")
    V = proposal_velocity.to(P.dtype).contiguous()
    I = initial_position.to(P.dtype).contiguous()
    D = None if alpha2_tangent is None else alpha2_tangent.to(P.dtype).contiguous()
    acc = acceptance_rate.to(torch.float64).contiguous()
    div = None if is_divergent is None else is_divergent.to(torch.uint8).contiguous()
    lib = L.lib()
    nbytes = int(lib.gj_chees_workspace_size(C, d))
    if workspace is None or workspace.numel() * workspace.element_size() < nbytes:
        workspace = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=P.device)
    out = torch.empty(3, dtype=torch.float64, device=P.device)
    L.check(lib.gj_chees_statistics(prec, C, d, L.ptr(P), L.ptr(V), L.ptr(I), L.ptr(D), L.ptr(acc),
                                    L.ptr(div), L.ptr(workspace), L.ptr(out),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    h, g, ga = out.tolist()
    return ChEESStatistics(h, g, ga)


# ---------------------------------------------------------------------------
# dynamic kernels (number of steps drawn per transition)
# ---------------------------------------------------------------------------
class DynamicRMHMCState(NamedTuple):
    """``rmhmc/rmhmc.py:44-55``."""

    position: Any
    logdensity: Any
    logdensity_grad: Any
    random_generator_arg: Any


class DynamicLMCState(NamedTuple):
    """``lmcmc/lmc.py`` / ``lmcmonge/lmc.py`` dynamic states."""

    position: Any
    logdensity: Any
    logdensity_grad: Any
    volume_adjustment: Any
    random_generator_arg: Any


_SAMPLERS = {"rmhmc": rmhmc, "lmc": lmc, "lmcmonge": lmcmonge}


def _random_steps(arg):
    g = torch.Generator()
    g.manual_seed(int(arg))
    return int(torch.randint(1, 10, (1,), generator=g))


class _Dynamic:
    """A base kernel whose number of integration steps comes from
    ``integration_steps_fn(random_generator_arg, **kwargs)``; all chains of a
    call share the state's counter, as under the reference's ``vmap`` with
    one initial argument."""

    dynamics = "rmhmc"

    @classmethod
    def init(cls, position, target, random_generator_arg=0):
        base = _SAMPLERS[cls.dynamics].init(position, target)
        if cls.dynamics == "rmhmc":
            return DynamicRMHMCState(*base, random_generator_arg)
        return DynamicLMCState(*base, random_generator_arg)

    @classmethod
    def build_kernel(cls, next_random_arg_fn: Callable = lambda a: a + 1,
                     integration_steps_fn: Callable = _random_steps, **kernel_options):
        base = _SAMPLERS[cls.dynamics].build_kernel(**kernel_options)
        lmc_like = cls.dynamics != "rmhmc"

        def kernel(rng_key, state, target, step_size, *, alpha2=0.0, inverse_mass_matrix=None,
                   **integration_steps_kwargs):
            n = int(integration_steps_fn(state.random_generator_arg, **integration_steps_kwargs))
            if lmc_like:
                inner = LMCState(state.position, state.logdensity, state.logdensity_grad,
                                 state.volume_adjustment)
            else:
                inner = RMHMCState(state.position, state.logdensity, state.logdensity_grad)
            kw = {}
            if cls.dynamics == "lmcmonge":
                kw = {"alpha2": alpha2, "inverse_mass_matrix": inverse_mass_matrix}
            new, info = base(rng_key, inner, target, step_size, n, **kw)
            nxt = next_random_arg_fn(state.random_generator_arg)
            return type(state)(*new, nxt), info

        return kernel


class dynamic_rmhmc(_Dynamic):
    """``rmhmc/rmhmc.py:314-373``."""

    dynamics = "rmhmc"


class dynamic_lmc(_Dynamic):
    """``lmcmc/lmc.py`` ``dynamic_lmc``."""

    dynamics = "lmc"


class dynamic_lmcmonge(_Dynamic):
    """``lmcmonge/lmc.py`` ``dynamic_lmc``."""

    dynamics = "lmcmonge"


_DYNAMIC = {"rmhmc": dynamic_rmhmc, "lmc": dynamic_lmc, "lmcmonge": dynamic_lmcmonge}


class ChEESWarmupInfo(NamedTuple):
    """Per warm-up step (the reference's ``AdaptationInfo`` keeps the full
    states; here the scalars that describe the step)."""

    adaptation_state: ChEESAdaptationState
    num_integration_steps: int
    statistics: ChEESStatistics


# ---------------------------------------------------------------------------
# the adaptation loop
# ---------------------------------------------------------------------------
def _chees(target, num_chains, dynamics, *, jitter_generator, jitter_amount,
           target_acceptance_rate, decay_rate, inverse_mass_matrix=None, alpha2=1.0,
           update_alpha=False, kernel_options=None):
    dyn = _DYNAMIC[dynamics]
    kernel_options = dict(kernel_options or {})

    def run(rng_key, positions, step_size: float, optim: GradientTransformation,
            num_steps: int = 1000, *, max_sampling_steps: int = 1000, draws=None):
        q = torch.as_tensor(positions)
        if q.shape[0] != num_chains:
            raise ValueError("initial `positions` leading dimension must be equal to "
                             "the `num_chains`")
        if jitter_generator is not None:
            def jitter_gn(arg):
                return jitter_generator(arg) * jitter_amount + (1.0 - jitter_amount)
        else:
            max_bits = math.ceil(math.log2(num_steps + max_sampling_steps))

            def jitter_gn(i):
                return halton_sequence(i, max_bits) * jitter_amount + (1.0 - jitter_amount)

        def next_random_arg_fn(i):
            return i + 1

        def integration_steps_fn(arg, trajectory_length_adjusted):
            return int(math.ceil(jitter_gn(arg) * trajectory_length_adjusted))

        kernel = dyn.build_kernel(next_random_arg_fn, integration_steps_fn, **kernel_options)
        states = dyn.init(q, target, 0)
        s = chees_init(0, float(step_size), optim, alpha2)
        gen = None
        if draws is None:
            gen = torch.Generator(device=target.device)
            gen.manual_seed(int(rng_key))
        im = None
        if inverse_mass_matrix is not None:
            im = torch.as_tensor(inverse_mass_matrix).to(device=target.device, dtype=target.dtype)
        alpha2_fix = bool(kernel_options.get("alpha2_fix", False))
        C, d = states.position.shape
        work = None
        history = []
        for i in range(num_steps):
            key = gen if draws is None else draws[i]
            z, u = Kernel.draws(key, C, d, target)
            T_adj = s.trajectory_length / s.step_size
            n = integration_steps_fn(states.random_generator_arg, T_adj)
            extra = {}
            if dynamics == "lmcmonge":
                extra = {"alpha2": s.alpha2, "inverse_mass_matrix": im}
            new_states, info = kernel(Draws(z, u), states, target, s.step_size,
                                      trajectory_length_adjusted=T_adj, **extra)
            if work is None:
                nbytes = int(L.lib().gj_chees_workspace_size(C, d))
                work = torch.empty((nbytes + 7) // 8, dtype=torch.float64, device=target.device)
            tangent = None
            if update_alpha:  # ∂q_L/∂α² of the same transition (:469-519)
                _, tangent = lmcmonge_alpha2_tangent(target, states.position, z, s.step_size, n,
                                                     s.alpha2, im, alpha2_fix)
            stats = chees_statistics(info.proposal.position, info.proposal.velocity,
                                     states.position, info.acceptance_rate, info.is_divergent,
                                     alpha2_tangent=tangent, workspace=work)
            jit = jitter_gn(s.random_generator_arg)
            s = chees_update(s, stats, jit, optim, next_random_arg_fn, target_acceptance_rate,
                             decay_rate, update_alpha)
            history.append(ChEESWarmupInfo(s, n, stats))
            states = new_states
        T_adj = _exp(s.log_trajectory_length_moving_average - s.log_step_size_moving_average)
        parameters = {
            "step_size": _exp(s.log_step_size_moving_average),
            "next_random_arg_fn": next_random_arg_fn,
            "integration_steps_fn": lambda arg: integration_steps_fn(arg, T_adj),
        }
        if dynamics == "lmcmonge":
            parameters["alpha2"] = s.alpha2
            parameters["inverse_mass_matrix"] = inverse_mass_matrix
        return AdaptationResults(states, parameters), history

    return AdaptationAlgorithm(run)


def chees_adaptation(target, num_chains: int, *, jitter_generator: Optional[Callable] = None,
                     jitter_amount: float = 1.0,
                     target_acceptance_rate: float = OPTIMAL_TARGET_ACCEPTANCE_RATE,
                     decay_rate: float = 0.5, dynamics: str = "lmc",
                     **kernel_options) -> AdaptationAlgorithm:
    """``chees_adaptation_riemanian.py:234-465``: ``run(rng_key, positions,
    step_size, optim, num_steps=1000, *, max_sampling_steps=1000)`` returns
    ``(AdaptationResults(last_states, parameters), history)``; ``parameters``
    has the moving-average step size and ``integration_steps_fn`` with the
    adapted T/h, for ``dynamic_rmhmc`` / ``dynamic_lmc``.  ``kernel_options``
    go to the base kernel's ``build_kernel``."""
    if dynamics not in ("lmc", "rmhmc"):
        raise ValueError("dynamics must be 'lmc' or 'rmhmc'")
    return _chees(target, num_chains, dynamics, jitter_generator=jitter_generator,
                  jitter_amount=jitter_amount, target_acceptance_rate=target_acceptance_rate,
                  decay_rate=decay_rate, kernel_options=kernel_options)


def lmcmonge_chees_adaptation(target, inverse_mass_matrix, num_chains: int, *,
                              jitter_generator: Optional[Callable] = None,
                              jitter_amount: float = 1.0,
                              target_acceptance_rate: float = OPTIMAL_TARGET_ACCEPTANCE_RATE,
                              decay_rate: float = 0.5, update_alpha: bool = False,
                              alpha2: float = 0.001, **kernel_options) -> AdaptationAlgorithm:
    """``chees_adaptation_lmcmonge.py:322-568``: step size and trajectory
    length, and with ``update_alpha`` α² as well, starting from ``alpha2``
    (see the module docstring for the reference's own α² handling).  The
    returned ``parameters["alpha2"]`` is the adaptation state's α²."""
    return _chees(target, num_chains, "lmcmonge", jitter_generator=jitter_generator,
                  jitter_amount=jitter_amount, target_acceptance_rate=target_acceptance_rate,
                  decay_rate=decay_rate, inverse_mass_matrix=inverse_mass_matrix,
                  alpha2=float(alpha2), update_alpha=bool(update_alpha),
                  kernel_options=kernel_options)
