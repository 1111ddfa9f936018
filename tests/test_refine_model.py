"""The stopping rule of the refined position-iterate solves, on a float64 /
float32 NumPy model of their arithmetic (no GPU).

The device form (csrc/logreg_batched.cu: refined_solve_w32, refined_solve,
refine_verdict) factors G in float32, takes x₀ from the float32 solve, and
corrects x += G₃₂⁻¹(p − G·x), the residual in float64 from the float32 Gram
and the prior.  It stops when:

* the predicted size of the next correction ‖dx_k‖²/‖dx_{k−1}‖ is below
  2⁻⁴⁴‖x₀‖ (converged);
* a correction shrinks by less than half: converged when below 2⁻³⁶‖x₀‖
  (the float64 residual's rounding floor), failed above it;
* a correction is not finite, or eight of them do not converge (failed).

A failed chain is factored in float64.  The model restates that loop with
NumPy's float32 Cholesky and triangular solves, and checks three regimes:

* the benchmark's posterior (logistic regression N = 1000, d = 25, at
  Laplace draws): converged on the predicted-size test in at most two
  corrections, within 1e-12 of the float64 solve;
* spectra log-spaced over κ(G) = 1e4 and 1e5 at d = 64: converged, within
  1e-11 of the float64 solve;
* κ(G) = 1e8 and 1e9 at d = 25: failed (stalled above the floor, or the
  float32 factorisation broke down), so the float64 factorisation takes
  over.

In this model the fallback starts between κ(G) = 1e6 and 3e6 at d = 64:
there the corrections stall at about 1e-11 to 4e-11 relative, just above
2⁻³⁶.  Below that range the predicted-size test stops the loop first.
"""
import numpy as np
import pytest
from scipy.linalg import solve_triangular

from oracle import targets as OT
from tests.helpers import laplace_draws

K_MAX = 8


def refined_solve_model(gram32, prior, p):
    """(x, how, corrections) for G = gram32 + prior·I, the device's rule
    step by step (float32 norms relative to ‖x₀‖∞); how is "predicted" or
    "floor" (converged) or "factorisation", "not finite", "stalled",
    "too many" (failed)."""
    d = gram32.shape[0]
    G32 = (gram32 + np.float32(prior) * np.eye(d, dtype=np.float32)).astype(np.float32)
    G64 = gram32.astype(np.float64) + prior * np.eye(d)
    try:
        L = np.linalg.cholesky(G32)  # float32 LAPACK
    except np.linalg.LinAlgError:
        return None, "factorisation", 0
    if not np.all(np.isfinite(L)):
        return None, "factorisation", 0

    def solve32(r):
        y = solve_triangular(L, r.astype(np.float32), lower=True)
        return solve_triangular(L.T, y, lower=False).astype(np.float32)

    x = solve32(p).astype(np.float64)
    xn = np.float32(np.max(np.abs(x)))
    if xn == 0:
        return x, "predicted", 0
    pr = np.float32(1.0)
    for k in range(K_MAX):
        r = p - G64 @ x
        dx = solve32(r)
        if not np.all(np.isfinite(dx)):
            return x, "not finite", k + 1
        er = np.float32(np.max(np.abs(dx))) / xn
        if er * er <= np.float32(2.0 ** -44) * pr:
            return x + dx, "predicted", k + 1
        if er > np.float32(0.5) * pr:
            return x + dx, ("floor" if er <= np.float32(2.0 ** -36) else "stalled"), k + 1
        x = x + dx
        pr = er
    return x, "too many", K_MAX


CONVERGED = ("predicted", "floor")
FAILED = ("factorisation", "not finite", "stalled", "too many")


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_benchmark_metrics_converge_in_two_corrections():
    from geomjax_gb300.data import logreg_data

    X, y = logreg_data(1000, 25, seed=0)
    ot = OT.LogisticRegression(X, y)
    q = laplace_draws(ot, 64, seed=41)
    G = ot.metric(q)
    rng = np.random.default_rng(42)
    worst, most = 0.0, 0
    for c in range(len(q)):
        gram32 = (G[c] - np.eye(25) / ot.prior_var).astype(np.float32)
        p = rng.standard_normal(25) * 16.0  # |p| of the benchmark's momenta
        x, how, k = refined_solve_model(gram32, 1.0 / ot.prior_var, p)
        assert how == "predicted", (c, how)
        ref = np.linalg.solve(gram32.astype(np.float64) + np.eye(25) / ot.prior_var, p)
        worst = max(worst, _rel(x, ref))
        most = max(most, k)
    assert most <= 2, most
    assert worst < 1e-12, worst


def _ill_gram(d, kappa, seed):
    """A float32 Gram with eigenvalues log-spaced over kappa (the prior is
    added by the solve)."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((d, d)))
    w = np.logspace(0, -np.log10(kappa), d) * 100.0
    return ((Q * w) @ Q.T).astype(np.float32)


@pytest.mark.parametrize("kappa", [1e4, 1e5])
def test_moderately_conditioned_metrics_converge(kappa):
    rng = np.random.default_rng(43)
    for seed in range(8):
        gram32 = _ill_gram(64, kappa, seed)
        p = rng.standard_normal(64)
        x, how, k = refined_solve_model(gram32, 0.0, p)
        assert how in CONVERGED, (seed, how, k)
        ref = np.linalg.solve(gram32.astype(np.float64), p)
        assert _rel(x, ref) < 1e-11, (seed, _rel(x, ref))


@pytest.mark.parametrize("kappa", [1e8, 1e9])
def test_ill_conditioned_metrics_fall_back(kappa):
    rng = np.random.default_rng(44)
    for seed in range(4):
        _, how, _ = refined_solve_model(_ill_gram(25, kappa, seed), 0.0, rng.standard_normal(25))
        assert how in FAILED, (seed, how)
