"""Iterative NUTS with the Riemannian metric (float64, one chain at a time).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``rmhmc/nuts.py`` (``build_kernel`` :78-161, ``iterative_nuts_proposal``
:253-348) over ``mcmc/trajectory.py`` (``Trajectory`` :54-118,
``dynamic_progressive_integration`` :149-317, ``dynamic_multiplicative_expansion``
:517-668), ``mcmc/termination.py`` (``iterative_uturn_numpyro`` :30-119),
``mcmc/proposal.py`` (``proposal_from_energy_diff`` :87-121,
``progressive_uniform_sampling`` / ``progressive_biased_sampling`` :186-245)
and the generalized U-turn of ``rmhmc/metrics.py:76-118``.

Randomness: the reference splits its key for every direction, every step's
progressive sample and every merge.  Here one transition of one chain reads
uniforms ``u`` laid out as

* ``u[k]``                    the direction of expansion k (+1 iff u < 1/2),
* ``u[M + k]``                the biased merge of expansion k,
* ``u[2M + 2**k − 1 + j]``    step j (≥ 1) of expansion k,

M = max_num_doublings, 2M + 2**M − 1 uniforms in all; ``bernoulli(key, p)``
is ``u < p``.  Chains are independent: the batched entry point loops.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import rmhmc as R


def num_uniforms(max_num_doublings):
    return 2 * max_num_doublings + 2 ** max_num_doublings - 1


def _logaddexp(a, b):
    return float(np.logaddexp(a, b))


def _expit(x):
    return float(1.0 / (1.0 + np.exp(-x))) if x >= 0 else float(np.exp(x) / (1.0 + np.exp(x)))


@dataclass
class State:  # IntegratorState of one chain (rmhmc/integrators.py)
    q: np.ndarray
    p: np.ndarray
    v: np.ndarray
    ld: float
    g: np.ndarray


@dataclass
class Proposal:  # mcmc/proposal.py:23-38
    state: State
    energy: float
    weight: float
    sum_log_p_accept: float


@dataclass
class Traj:  # mcmc/trajectory.py:54-59
    left: State
    right: State
    p_sum: np.ndarray
    v_sum: np.ndarray
    n: int


def is_turning(m_left, m_right, m_sum, v_left, v_right, v_sum, criterion="euc"):
    """rmhmc/metrics.py:76-118."""
    if criterion == "euc":
        rho = v_sum
        return bool(v_left @ rho <= 0 or v_right @ rho <= 0)
    if criterion == "bet":
        rho = m_sum
        return bool(v_left @ rho <= 0 or v_right @ rho <= 0)
    if criterion == "riem":
        rho = v_sum
        return bool(m_left @ rho <= 0 or m_right @ rho <= 0)
    raise ValueError(criterion)


def leaf_idx_to_ckpt_idxs(n):
    """termination.py:78-93: idx_max = set bits of n >> 1, idx_min =
    idx_max − (trailing ones of n) + 1."""
    idx_max = bin(n >> 1).count("1")
    ones, m = 0, n
    while m & 1:
        m >>= 1
        ones += 1
    return idx_max - ones + 1, idx_max


class Termination:
    """iterative_uturn_numpyro (termination.py:30-119)."""

    def __init__(self, M, d):
        self.r = np.zeros((M, d))
        self.r_sum = np.zeros((M, d))
        self.v = np.zeros((M, d))
        self.v_sum = np.zeros((M, d))
        self.idx_min = 0
        self.idx_max = 0

    def update(self, r_sum, r, v_sum, v, step):
        lo, hi = leaf_idx_to_ckpt_idxs(step)
        if step % 2 == 0:
            self.r[hi], self.r_sum[hi], self.v[hi], self.v_sum[hi] = r, r_sum, v, v_sum
        self.idx_min, self.idx_max = lo, hi

    def turning(self, r_sum, r, v_sum, v, criterion):
        i = self.idx_max
        while i >= self.idx_min:
            sr = r_sum - self.r_sum[i] + self.r[i]
            sv = v_sum - self.v_sum[i] + self.v[i]
            if is_turning(self.r[i], r, sr, self.v[i], v, sv, criterion):
                return True
            i -= 1
        return False


def _step(target, s: State, h, integrator, tol, max_iters):
    """One integrator step; a metric that stops being positive definite
    gives a NaN state (JAX's solve and Cholesky return NaN where NumPy
    raises), which the energy difference turns into a divergence."""
    st = R.IntegratorState(s.q[None], s.p[None], s.v[None], np.array([s.ld]), s.g[None])
    try:
        with np.errstate(all="ignore"):
            new, _ = R.INTEGRATORS[integrator](target, st, h, tol=tol, max_iters=max_iters)
    except np.linalg.LinAlgError:
        nan = np.full_like(s.q, np.nan)
        return State(nan, nan.copy(), nan.copy(), float("nan"), nan.copy())
    return State(new.position[0], new.momentum[0], new.velocity[0], float(new.logdensity[0]),
                 new.logdensity_grad[0])


def _energy(target, s: State):
    """hmc_energy: −ℓ + K (mcmc/metrics.py:160-166)."""
    try:
        with np.errstate(all="ignore"):
            return -s.ld + float(R.kinetic_energy(target, s.q[None], s.p[None])[0])
    except np.linalg.LinAlgError:
        return float("nan")


def _from_energy_diff(H0, H1, state):
    """proposal.py:87-121."""
    w = H0 - H1
    if np.isnan(w):
        w = -np.inf
    return Proposal(state, H1, w, min(w, 0.0))


@dataclass
class NUTSInfo:
    momentum: np.ndarray
    is_divergent: bool
    is_turning: bool
    energy: float
    left: State
    right: State
    num_trajectory_expansions: int
    num_integration_steps: int
    acceptance_rate: float


def transition_one(target, q, ld, g, z, u, step_size, max_num_doublings=10, *,
                   integrator="implicit_midpoint", criterion="euc", tol=1e-6, max_iters=100,
                   divergence_threshold=1000.0):
    """One NUTS transition of one chain (rmhmc/nuts.py:112-159)."""
    M = max_num_doublings
    p = R.momentum_from_normals(target, q[None], z[None])[0]
    v = R.inverse_metric_vector_product(target, q[None], p[None])[0]
    s0 = State(q, p, v, float(ld), g)
    H0 = _energy(target, s0)
    proposal = Proposal(s0, H0, 0.0, -np.inf)
    traj = Traj(s0, s0, p.copy(), v.copy(), 0)
    term = Termination(M, q.shape[0])
    step = 0
    div = turning = False
    while step < M and not div and not turning:  # trajectory.py:560-565
        direction = 1 if u[step] < 0.5 else -1
        start = traj.right if direction > 0 else traj.left
        # dynamic_progressive_integration (trajectory.py:149-317)
        base = 2 * M + 2 ** step - 1
        cur = start
        sub_prop = None
        sub = Traj(start, start, start.p, start.v, 0)
        j = 0
        sub_div = sub_term = False
        while j < 2 ** step and not sub_term and not sub_div:
            new = _step(target, cur, direction * step_size, integrator, tol, max_iters)
            new_prop = _from_energy_diff(H0, _energy(target, new), new)
            sub_div = -new_prop.weight > divergence_threshold
            if j == 0:
                sub = Traj(new, new, new.p.copy(), new.v.copy(), 1)
                sub_prop = new_prop
            else:
                sub = Traj(sub.left, new, sub.p_sum + new.p, sub.v_sum + new.v, sub.n + 1)
                # progressive_uniform_sampling (proposal.py:186-212)
                acc = u[base + j] < _expit(new_prop.weight - sub_prop.weight)
                w = _logaddexp(sub_prop.weight, new_prop.weight)
                sl = _logaddexp(sub_prop.sum_log_p_accept, new_prop.sum_log_p_accept)
                sub_prop = Proposal(new if acc else sub_prop.state,
                                    new_prop.energy if acc else sub_prop.energy, w, sl)
            term.update(sub.p_sum, new.p, sub.v_sum, new.v, j)
            sub_term = term.turning(sub.p_sum, new.p, sub.v_sum, new.v, criterion)
            cur = new
            j += 1
        if direction < 0:
            sub = Traj(sub.right, sub.left, sub.p_sum, sub.v_sum, sub.n)
        # proposal update (trajectory.py:609-632)
        if sub_div or sub_term:
            proposal = Proposal(proposal.state, proposal.energy, proposal.weight,
                                _logaddexp(proposal.sum_log_p_accept, sub_prop.sum_log_p_accept))
        else:  # progressive_biased_sampling (proposal.py:215-245)
            with np.errstate(over="ignore"):
                pa = min(float(np.exp(sub_prop.weight - proposal.weight)), 1.0)
            acc = u[M + step] < pa
            w = _logaddexp(proposal.weight, sub_prop.weight)
            sl = _logaddexp(proposal.sum_log_p_accept, sub_prop.sum_log_p_accept)
            proposal = Proposal(sub_prop.state if acc else proposal.state,
                                sub_prop.energy if acc else proposal.energy, w, sl)
        left_t, right_t = (traj, sub) if direction > 0 else (sub, traj)
        traj = Traj(left_t.left, right_t.right, left_t.p_sum + right_t.p_sum,
                    left_t.v_sum + right_t.v_sum, left_t.n + right_t.n)
        whole = is_turning(traj.left.p, traj.right.p, traj.p_sum, traj.left.v, traj.right.v,
                           traj.v_sum, criterion)
        div = sub_div
        turning = sub_term or whole
        step += 1
    acc_rate = float(np.exp(proposal.sum_log_p_accept) / traj.n)
    info = NUTSInfo(p, div, turning, proposal.energy, traj.left, traj.right, step, traj.n,
                    acc_rate)
    return proposal.state, info


def kernel(target, state, z, u, step_size, max_num_doublings=10, **kw):
    """All chains of an ``rmhmc.RMHMCState``; ``u``: [C, num_uniforms(M)]."""
    C = state.position.shape[0]
    qs, lds, gs, infos = [], [], [], []
    for c in range(C):
        s, info = transition_one(target, state.position[c], state.logdensity[c],
                                 state.logdensity_grad[c], z[c], u[c], step_size,
                                 max_num_doublings, **kw)
        qs.append(s.q)
        lds.append(s.ld)
        gs.append(s.g)
        infos.append(info)
    return R.RMHMCState(np.array(qs), np.array(lds), np.array(gs)), infos
