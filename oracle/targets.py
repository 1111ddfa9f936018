"""Target families for the oracle (float64, batched over chains).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

The reference receives targets as user Python callables ``logdensity_fn(θ)``
and ``metric_fn(θ)`` and differentiates them with JAX
(``rmhmc/integrators.py:111-114``, ``util.py:120-121`` HVP,
``lmcmc/metrics.py:165`` jacfwd).  The device build registers three
families with analytic operators instead; the oracle states the same
operators analytically and the tests check them against central finite
differences.

Every target exposes, for positions ``q[C, d]``:

* ``logdensity(q) -> [C]`` and ``grad(q) -> [C, d]``
* ``hvp(q, u) -> [C, d]`` (Hessian of the log density times ``u``,
  the reference's ``jvp(grad f)``, ``util.py:120-121``)
* ``metric(q)`` -> ``[C, d]`` (diagonal) or ``[C, d, d]`` (dense)
* ``dmetric(q)`` -> ``[C, d, k]`` (diagonal: ∂G_a/∂q_k) or ``[C, d, d, k]``
  (dense: ∂G_ab/∂q_k), the reference's ``jax.jacfwd(metric_fn)`` layout
  (``lmcmc/metrics.py:165``).
"""
from __future__ import annotations

import numpy as np

LOG2PI = np.log(2.0 * np.pi)


def _norm_logpdf(x, loc, scale):
    z = (x - loc) / scale
    return -0.5 * z * z - np.log(scale) - 0.5 * LOG2PI


class Funnel:
    """Neal's funnel, ``examples/funnel/main.py:28-54``.

    v = θ[D-1] ~ N(0, σ²), x_i = θ[i] | v ~ N(0, e^v) for i < D-1 (the
    reference puts v LAST, ``main.py:35-39``).

    ``metric="diag"``: expected Fisher information diag(e^{-v} for x,
    1/σ² + (D-1)/2 for v) — the position-dependent diagonal metric of the
    plain FP64 configuration, mapped onto the reference's ordering.
    ``metric="pullback"``: the dense pull-back metric J⁻ᵀJ⁻¹ of
    ``main.py:41-54``.
    """

    family = "funnel"

    def __init__(self, D: int = 2, sigma: float = 3.0, metric: str = "diag"):
        self.D = D
        self.dim = D
        self.sigma = float(sigma)
        self.metric_kind = metric

    # --- log density (main.py:35-39) -------------------------------------
    def logdensity(self, q):
        v = q[:, -1]
        x = q[:, :-1]
        return _norm_logpdf(v, 0.0, self.sigma) + np.sum(
            _norm_logpdf(x, 0.0, np.exp(0.5 * v)[:, None]), axis=1
        )

    def grad(self, q):
        v = q[:, -1]
        x = q[:, :-1]
        ev = np.exp(-v)
        g = np.empty_like(q)
        g[:, :-1] = -x * ev[:, None]
        g[:, -1] = -v / self.sigma**2 - 0.5 * (self.D - 1) + 0.5 * ev * np.sum(x * x, axis=1)
        return g

    def hvp(self, q, u):
        v = q[:, -1]
        x = q[:, :-1]
        ev = np.exp(-v)
        out = np.empty_like(q)
        out[:, :-1] = ev[:, None] * (-u[:, :-1] + x * u[:, -1:])
        out[:, -1] = ev * np.sum(x * u[:, :-1], axis=1) + (
            -1.0 / self.sigma**2 - 0.5 * ev * np.sum(x * x, axis=1)
        ) * u[:, -1]
        return out

    # --- metrics ----------------------------------------------------------
    @property
    def is_diagonal(self):
        return self.metric_kind == "diag"

    def metric(self, q):
        v = q[:, -1]
        x = q[:, :-1]
        ev = np.exp(-v)
        C, D = q.shape
        if self.metric_kind == "diag":
            G = np.empty_like(q)
            G[:, :-1] = ev[:, None]
            G[:, -1] = 1.0 / self.sigma**2 + 0.5 * (D - 1)
            return G
        # pull-back J^{-T} J^{-1}, main.py:41-54
        G = np.zeros((C, D, D))
        idx = np.arange(D - 1)
        G[:, idx, idx] = ev[:, None]
        G[:, :-1, -1] = -0.5 * ev[:, None] * x
        G[:, -1, :-1] = -0.5 * ev[:, None] * x
        G[:, -1, -1] = 0.25 * ev * np.sum(x * x, axis=1) + 1.0 / self.sigma**2
        return G

    def dmetric(self, q):
        v = q[:, -1]
        x = q[:, :-1]
        ev = np.exp(-v)
        C, D = q.shape
        if self.metric_kind == "diag":
            dG = np.zeros((C, D, D))
            dG[:, :-1, -1] = -ev[:, None]
            return dG
        dG = np.zeros((C, D, D, D))
        idx = np.arange(D - 1)
        # derivative w.r.t. x_k (k < D-1)
        dG[:, idx, -1, idx] = -0.5 * ev[:, None]
        dG[:, -1, idx, idx] = -0.5 * ev[:, None]
        dG[:, -1, -1, :-1] = 0.5 * ev[:, None] * x
        # derivative w.r.t. v
        dG[:, idx, idx, -1] = -ev[:, None]
        dG[:, :-1, -1, -1] = 0.5 * ev[:, None] * x
        dG[:, -1, :-1, -1] = 0.5 * ev[:, None] * x
        dG[:, -1, -1, -1] = -0.25 * ev * np.sum(x * x, axis=1)
        return dG


class LogisticRegression:
    """Bayesian logistic regression with the dense Fisher metric.

    Not in the reference (its shape is implied by ``metric_fn`` in
    ``rmhmc/metrics.py:42-127`` and ``lmcmc/metrics.py:42-219``).
    ℓ(β) = Σ_n [y_n a_n − log(1+e^{a_n})] + log N(β; 0, s²I), a = Xβ.
    G(β) = XᵀΛX + I/s², Λ = σ(a)(1−σ(a)).
    ∂G/∂β_k = Xᵀ diag(Λ' ⊙ X[:, k]) X, Λ' = σ(1−σ)(1−2σ).
    """

    family = "logistic_regression"
    is_diagonal = False
    # ∂_kG_ij = Σ_n Λ'_n x_ni x_nj x_nk is symmetric in (i, j, k)
    dmetric_fully_symmetric = True

    def __init__(self, X, y, prior_var: float = 100.0):
        self.X = np.asarray(X, dtype=np.float64)
        self.y = np.asarray(y, dtype=np.float64)
        self.N, self.dim = self.X.shape
        self.prior_var = float(prior_var)

    def _a(self, q):
        return q @ self.X.T  # [C, N]

    def logdensity(self, q):
        a = self._a(q)
        lik = np.sum(self.y * a - np.logaddexp(0.0, a), axis=1)
        prior = -0.5 * np.sum(q * q, axis=1) / self.prior_var - 0.5 * self.dim * (
            LOG2PI + np.log(self.prior_var)
        )
        return lik + prior

    def grad(self, q):
        s = _sigmoid(self._a(q))
        return (self.y - s) @ self.X - q / self.prior_var

    def hvp(self, q, u):
        s = _sigmoid(self._a(q))
        lam = s * (1.0 - s)
        return -((lam * (u @ self.X.T)) @ self.X) - u / self.prior_var

    def metric(self, q):
        s = _sigmoid(self._a(q))
        lam = s * (1.0 - s)
        # Σ_n Λ_cn x_n x_nᵀ per chain, as one matmul per chain
        G = np.matmul(np.swapaxes(lam[:, :, None] * self.X[None], 1, 2), self.X[None])
        G += np.eye(self.dim)[None] / self.prior_var
        return G

    def dmetric(self, q):
        s = _sigmoid(self._a(q))
        lamp = s * (1.0 - s) * (1.0 - 2.0 * s)
        return np.einsum("cn,ni,nj,nk->cijk", lamp, self.X, self.X, self.X)

    # structured contractions (avoid the d³ tensor for realistic sizes)
    def metric_trace_quad(self, q, Ginv, u):
        """Return tr(G⁻¹∂_kG) and uᵀ∂_kG u for every k ([C, d] each)."""
        s = _sigmoid(self._a(q))
        lamp = s * (1.0 - s) * (1.0 - 2.0 * s)
        w = np.sum(np.matmul(self.X[None], Ginv) * self.X[None], axis=2)  # x_nᵀ G⁻¹ x_n
        xu = u @ self.X.T  # [C, N]
        tr = (lamp * w) @ self.X
        quad = (lamp * xu * xu) @ self.X
        return tr, quad

    def dmetric_vec(self, q, v):
        """Σ_i v_i ∂_i G  ([C, d, d]); ∂G is fully symmetric for this family."""
        s = _sigmoid(self._a(q))
        lamp = s * (1.0 - s) * (1.0 - 2.0 * s)
        xv = v @ self.X.T
        wgt = lamp * xv
        return np.matmul(np.swapaxes(wgt[:, :, None] * self.X[None], 1, 2), self.X[None])


class HierarchicalGaussian:
    """Hierarchical Gaussian (centred), global parameters LAST like the funnel.

    θ = [θ_1..θ_J, μ, v]; y_j ~ N(θ_j, σ_j²), θ_j ~ N(μ, e^v),
    μ ~ N(0, s_μ²), v ~ N(0, s_v²).  Not in the reference; registered so the
    dense-metric paths have a funnel-shaped posterior with an arrowhead
    Fisher metric:
      G_{θjθj} = 1/σ_j² + e^{-v}, G_{θjμ} = −e^{-v}, G_{μμ} = J e^{-v} + 1/s_μ²,
      G_{vv} = J/2 + 1/s_v², all other entries 0.
    """

    family = "hierarchical_gaussian"
    is_diagonal = False

    def __init__(self, y, sigma, mu_scale: float = 5.0, v_scale: float = 2.0):
        self.y = np.asarray(y, dtype=np.float64)
        self.sig = np.asarray(sigma, dtype=np.float64)
        self.J = self.y.shape[0]
        self.dim = self.J + 2
        self.mu_scale = float(mu_scale)
        self.v_scale = float(v_scale)

    def logdensity(self, q):
        th, mu, v = q[:, : self.J], q[:, self.J], q[:, self.J + 1]
        out = np.sum(_norm_logpdf(self.y[None], th, self.sig[None]), axis=1)
        out += np.sum(_norm_logpdf(th, mu[:, None], np.exp(0.5 * v)[:, None]), axis=1)
        out += _norm_logpdf(mu, 0.0, self.mu_scale) + _norm_logpdf(v, 0.0, self.v_scale)
        return out

    def grad(self, q):
        J = self.J
        th, mu, v = q[:, :J], q[:, J], q[:, J + 1]
        ev = np.exp(-v)
        r = th - mu[:, None]
        g = np.empty_like(q)
        g[:, :J] = (self.y[None] - th) / self.sig[None] ** 2 - r * ev[:, None]
        g[:, J] = np.sum(r, axis=1) * ev - mu / self.mu_scale**2
        g[:, J + 1] = 0.5 * ev * np.sum(r * r, axis=1) - 0.5 * J - v / self.v_scale**2
        return g

    def hvp(self, q, u):
        J = self.J
        th, mu, v = q[:, :J], q[:, J], q[:, J + 1]
        ev = np.exp(-v)
        r = th - mu[:, None]
        ut, um, uv = u[:, :J], u[:, J], u[:, J + 1]
        out = np.empty_like(q)
        out[:, :J] = (
            -(1.0 / self.sig[None] ** 2 + ev[:, None]) * ut
            + ev[:, None] * um[:, None]
            + r * ev[:, None] * uv[:, None]
        )
        out[:, J] = ev * np.sum(ut, axis=1) + (-J * ev - 1.0 / self.mu_scale**2) * um - ev * np.sum(r, axis=1) * uv
        out[:, J + 1] = (
            ev * np.sum(r * ut, axis=1)
            - ev * np.sum(r, axis=1) * um
            + (-0.5 * ev * np.sum(r * r, axis=1) - 1.0 / self.v_scale**2) * uv
        )
        return out

    def metric(self, q):
        J = self.J
        v = q[:, J + 1]
        ev = np.exp(-v)
        C = q.shape[0]
        G = np.zeros((C, J + 2, J + 2))
        idx = np.arange(J)
        G[:, idx, idx] = 1.0 / self.sig[None] ** 2 + ev[:, None]
        G[:, idx, J] = -ev[:, None]
        G[:, J, idx] = -ev[:, None]
        G[:, J, J] = J * ev + 1.0 / self.mu_scale**2
        G[:, J + 1, J + 1] = 0.5 * J + 1.0 / self.v_scale**2
        return G

    def dmetric(self, q):
        J = self.J
        v = q[:, J + 1]
        ev = np.exp(-v)
        C = q.shape[0]
        dG = np.zeros((C, J + 2, J + 2, J + 2))
        idx = np.arange(J)
        dG[:, idx, idx, J + 1] = -ev[:, None]
        dG[:, idx, J, J + 1] = ev[:, None]
        dG[:, J, idx, J + 1] = ev[:, None]
        dG[:, J, J, J + 1] = -J * ev
        return dG


class IdentityMetric:
    """Wrap a target with G = I (``tests/test_samplers.py:25,37``)."""

    is_diagonal = False

    def __init__(self, base):
        self.base = base
        self.dim = base.dim
        self.family = base.family

    def logdensity(self, q):
        return self.base.logdensity(q)

    def grad(self, q):
        return self.base.grad(q)

    def hvp(self, q, u):
        return self.base.hvp(q, u)

    def metric(self, q):
        return np.broadcast_to(np.eye(self.dim), (q.shape[0], self.dim, self.dim)).copy()

    def dmetric(self, q):
        return np.zeros((q.shape[0], self.dim, self.dim, self.dim))


def _sigmoid(a):
    return 0.5 * (1.0 + np.tanh(0.5 * a))


def make_logreg_data(N: int, d: int, seed: int = 0, dtype=np.float32):
    """Synthetic logistic-regression data: X iid N(0,1), β*~N(0,I),
    y ~ Bernoulli(σ(Xβ*)), numpy PCG64 seeded.  X is rounded to ``dtype``
    (FP32 on the device) and returned as float64 holding those values."""
    rng = np.random.Generator(np.random.PCG64(seed))
    X = rng.standard_normal((N, d)).astype(dtype).astype(np.float64)
    beta = rng.standard_normal(d)
    p = _sigmoid(X @ beta)
    y = (rng.random(N) < p).astype(np.float64)
    return X, y


def make_hier_data(J: int, seed: int = 0):
    rng = np.random.Generator(np.random.PCG64(seed))
    sigma = rng.uniform(5.0, 15.0, J).astype(np.float32).astype(np.float64)
    y = (rng.standard_normal(J) * 10.0).astype(np.float32).astype(np.float64)
    return y, sigma
