"""Iterative NUTS (float64, one chain at a time) with the RMHMC, dense LMC or
LMC-Monge dynamics.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``rmhmc/nuts.py`` (``build_kernel`` :78-161, ``iterative_nuts_proposal``
:253-348), ``lmcmc/nuts.py`` and ``lmcmonge/nuts.py`` (the same tree over
the lan integrators and the LMC energies; LMC-Monge returns the gradient
de-normalised, ``lmcmonge/nuts.py:196-203``) over ``mcmc/trajectory.py`` (``Trajectory`` :54-118,
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
class State:  # one chain's integrator state and its U-turn vectors
    inner: object       # the dynamics' own (batched, C = 1) state
    m: np.ndarray       # momentum
    u: np.ndarray       # velocity
    q: np.ndarray
    ld: float


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


def _nan_like(s: State):
    nan = np.full_like(s.q, np.nan)
    return State(None, nan, nan.copy(), nan.copy(), float("nan"))


class RmDynamics:
    """RMHMC: IntegratorState (q, p, G⁻¹p, ℓ, ∇ℓ), energy −ℓ + K."""

    def __init__(self, target, integrator="implicit_midpoint", tol=1e-6, max_iters=100, **_):
        self.t, self.integ, self.tol, self.max_iters = target, integrator, tol, max_iters

    def _wrap(self, st):
        return State(st, st.momentum[0], st.velocity[0], st.position[0], float(st.logdensity[0]))

    def start(self, q, ld, g, J, z):
        p = R.momentum_from_normals(self.t, q[None], z[None])
        v = R.inverse_metric_vector_product(self.t, q[None], p)
        return self._wrap(R.IntegratorState(q[None], p, v, np.array([ld]), g[None]))

    def step(self, s, h):
        new, _ = R.INTEGRATORS[self.integ](self.t, s.inner, h, tol=self.tol,
                                           max_iters=self.max_iters)
        return self._wrap(new)

    def energy(self, s):  # hmc_energy (mcmc/metrics.py:160-166)
        return -s.ld + float(R.kinetic_energy(self.t, s.inner.position, s.inner.momentum)[0])

    def out(self, s):
        return s.q, s.ld, s.inner.logdensity_grad[0], 0.0


class LmcDynamics:
    """dense LMC: IntegratorState (q, Gv, v, ℓ, ∇ℓ, J), energy −ℓ + K − J."""

    def __init__(self, target, **_):
        self.t = target

    def _wrap(self, st):
        return State(st, st.momentum[0], st.velocity[0], st.position[0], float(st.logdensity[0]))

    def start(self, q, ld, g, J, z):
        from . import lmc as Lm

        v = Lm.velocity(self.t, q[None], z[None])
        mom = Lm.metric_vector_product(self.t, q[None], v)
        return self._wrap(Lm.IntegratorState(q[None], mom, v, np.array([ld]), g[None],
                                             np.array([J])))

    def step(self, s, h):
        from . import lmc as Lm

        return self._wrap(Lm.lan_step(self.t, s.inner, h))

    def energy(self, s):
        from . import lmc as Lm

        return float(Lm.energy(self.t, s.inner)[0])

    def out(self, s):
        return s.q, s.ld, s.inner.logdensity_grad[0], float(s.inner.volume_adjustment[0])


class MongeDynamics:
    """LMC-Monge: RiemannianIntegratorState, energy −ℓ + K − J."""

    def __init__(self, target, alpha2=0.001, inverse_mass_matrix=None, alpha2_fix=False, **_):
        self.t, self.a2, self.fix = target, alpha2, alpha2_fix
        self.im = (np.ones(target.dim) if inverse_mass_matrix is None
                   else np.asarray(inverse_mass_matrix, dtype=np.float64))
        self.mass = 1.0 / self.im

    def _wrap(self, st):
        return State(st, st.momentum[0], st.velocity[0], st.position[0], float(st.logdensity[0]))

    def start(self, q, ld, g, J, z):
        from . import lmcmonge as Mo

        a2, im = self.a2, self.im
        q1, g1 = q[None], g[None]
        L = Mo.normalizing_constant(a2, im, g1)
        sL = np.sqrt(L)[:, None]
        g_n = g1 / sL
        dl_ig = im * g_n
        Hdl_ig = self.t.hvp(q1, dl_ig) / sL
        v = Mo.velocity_dense(a2, im, dl_ig, z[None])
        mom = Mo.metric_vector_product(v, a2, g1, L, self.mass)
        hv_n = self.t.hvp(q1, v) / sL
        return self._wrap(Mo.MongeState(a2, q1, mom, v, np.array([ld]), g_n, dl_ig, Hdl_ig,
                                        im * Hdl_ig, hv_n, L, np.array([J])))

    def step(self, s, h):
        from . import lmcmonge as Mo

        return self._wrap(Mo.lan_step(self.t, s.inner, h, self.im, self.mass, self.fix))

    def energy(self, s):
        from . import lmcmonge as Mo

        return float(Mo.energy(s.inner, self.mass)[0])

    def out(self, s):
        st = s.inner
        g = st.logdensity_grad_norm[0] * np.sqrt(st.determinant_metric[0])
        return s.q, s.ld, g, float(st.volume_adjustment[0])


DYNAMICS = {"rmhmc": RmDynamics, "lmc": LmcDynamics, "lmcmonge": MongeDynamics}


def _safe_step(dyn, s, h):
    """One integrator step; a metric that stops being positive definite
    gives a NaN state (JAX's solve and Cholesky return NaN where NumPy
    raises), which the energy difference turns into a divergence."""
    try:
        with np.errstate(all="ignore"):
            return dyn.step(s, h)
    except np.linalg.LinAlgError:
        return _nan_like(s)


def _safe_energy(dyn, s):
    if s.inner is None:
        return float("nan")
    try:
        with np.errstate(all="ignore"):
            return dyn.energy(s)
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


def transition_one(target, q, ld, g, z, u, step_size, max_num_doublings=10, *, dynamics="rmhmc",
                   criterion="euc", divergence_threshold=1000.0, volume_adjustment=0.0, **dyn_kw):
    """One NUTS transition of one chain (rmhmc/nuts.py:112-159 and its LMC
    twins); ``dyn_kw`` configures the dynamics (integrator, tol, max_iters
    for RMHMC; alpha2, inverse_mass_matrix, alpha2_fix for LMC-Monge).
    Returns ((q, ℓ, ∇ℓ, J) of the sampled proposal, NUTSInfo)."""
    dyn = DYNAMICS[dynamics](target, **dyn_kw)
    M = max_num_doublings
    s0 = dyn.start(q, float(ld), g, float(volume_adjustment), z)
    H0 = dyn.energy(s0)
    proposal = Proposal(s0, H0, 0.0, -np.inf)
    traj = Traj(s0, s0, s0.m.copy(), s0.u.copy(), 0)
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
        sub = None
        j = 0
        sub_div = sub_term = False
        while j < 2 ** step and not sub_term and not sub_div:
            new = _safe_step(dyn, cur, direction * step_size)
            new_prop = _from_energy_diff(H0, _safe_energy(dyn, new), new)
            sub_div = -new_prop.weight > divergence_threshold
            if j == 0:
                sub = Traj(new, new, new.m.copy(), new.u.copy(), 1)
                sub_prop = new_prop
            else:
                sub = Traj(sub.left, new, sub.p_sum + new.m, sub.v_sum + new.u, sub.n + 1)
                # progressive_uniform_sampling (proposal.py:186-212)
                acc = u[base + j] < _expit(new_prop.weight - sub_prop.weight)
                w = _logaddexp(sub_prop.weight, new_prop.weight)
                sl = _logaddexp(sub_prop.sum_log_p_accept, new_prop.sum_log_p_accept)
                sub_prop = Proposal(new if acc else sub_prop.state,
                                    new_prop.energy if acc else sub_prop.energy, w, sl)
            term.update(sub.p_sum, new.m, sub.v_sum, new.u, j)
            sub_term = term.turning(sub.p_sum, new.m, sub.v_sum, new.u, criterion)
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
        whole = is_turning(traj.left.m, traj.right.m, traj.p_sum, traj.left.u, traj.right.u,
                           traj.v_sum, criterion)
        div = sub_div
        turning = sub_term or whole
        step += 1
    acc_rate = float(np.exp(proposal.sum_log_p_accept) / traj.n)
    info = NUTSInfo(s0.m, div, turning, proposal.energy, traj.left, traj.right, step, traj.n,
                    acc_rate)
    return dyn.out(proposal.state), info


def kernel(target, state, z, u, step_size, max_num_doublings=10, *, dynamics="rmhmc", **kw):
    """All chains of an ``rmhmc.RMHMCState`` (or an LMC state with a volume
    adjustment); ``u``: [C, num_uniforms(M)].  Returns the new state (the
    same type) and the per-chain infos."""
    C = state.position.shape[0]
    vol = getattr(state, "volume_adjustment", None)
    outs, infos = [], []
    for c in range(C):
        o, info = transition_one(target, state.position[c], state.logdensity[c],
                                 state.logdensity_grad[c], z[c], u[c], step_size,
                                 max_num_doublings, dynamics=dynamics,
                                 volume_adjustment=0.0 if vol is None else vol[c], **kw)
        outs.append(o)
        infos.append(info)
    q = np.array([o[0] for o in outs])
    ld = np.array([o[1] for o in outs])
    g = np.array([o[2] for o in outs])
    if vol is None:
        return R.RMHMCState(q, ld, g), infos
    return type(state)(q, ld, g, np.array([o[3] for o in outs])), infos
