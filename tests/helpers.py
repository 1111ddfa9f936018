"""Shared builders for the parity tests: the same target spec as an oracle
(float64 NumPy) object and as a device (geomjax_gb300) object."""
from __future__ import annotations

import numpy as np

from oracle import targets as OT


def oracle_target(kind, **kw):
    if kind == "funnel":
        return OT.Funnel(D=kw.get("D", 2), sigma=kw.get("sigma", 3.0), metric=kw.get("metric", "diag"))
    if kind == "logreg":
        X, y = OT.make_logreg_data(kw["N"], kw["d"], seed=kw.get("seed", 0))
        t = OT.LogisticRegression(X, y, prior_var=kw.get("prior_var", 100.0))
        if kw.get("metric") == "identity":
            return OT.IdentityMetric(t)
        return t
    if kind == "hier":
        y, s = OT.make_hier_data(kw["J"], seed=kw.get("seed", 0))
        t = OT.HierarchicalGaussian(y, s)
        if kw.get("metric") == "identity":
            return OT.IdentityMetric(t)
        return t
    raise ValueError(kind)


def device_target(kind, precision, **kw):
    import geomjax_gb300 as gj

    if kind == "funnel":
        return gj.funnel(D=kw.get("D", 2), sigma=kw.get("sigma", 3.0), metric=kw.get("metric", "diag"),
                         precision=precision)
    if kind == "logreg":
        X, y = OT.make_logreg_data(kw["N"], kw["d"], seed=kw.get("seed", 0))
        return gj.logistic_regression(X, y, prior_var=kw.get("prior_var", 100.0),
                                      metric="identity" if kw.get("metric") == "identity" else "fisher",
                                      precision=precision)
    if kind == "hier":
        y, s = OT.make_hier_data(kw["J"], seed=kw.get("seed", 0))
        return gj.hierarchical_gaussian(y, s, metric="identity" if kw.get("metric") == "identity" else "fisher",
                                        precision=precision)
    raise ValueError(kind)


def start_positions(dim, C, seed=0, scale=0.5):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((C, dim)) * scale


def normals(C, dim, seed, dtype=np.float64):
    """Host-drawn draws; for the mixed form z is rounded to float32 first so
    the oracle sees exactly the device's inputs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    z = rng.standard_normal((C, dim)).astype(dtype).astype(np.float64)
    u = rng.random(C)
    return z, u


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.max(np.abs(a - b) / (np.abs(b) + 1.0))


def laplace_draws(ot, C, seed, newton_iters=25):
    """C positions drawn from the Laplace approximation of a logistic-regression
    posterior: the mode by Newton steps β ← β + G(β)⁻¹∇ℓ(β) (the Fisher metric
    is the negative Hessian of the log density for this family), then
    β ~ N(mode, G(mode)⁻¹).  Chains started there are in the typical set."""
    b = np.zeros((1, ot.dim))
    for _ in range(newton_iters):
        b = b + np.linalg.solve(ot.metric(b), ot.grad(b)[..., None])[..., 0]
    L = np.linalg.cholesky(ot.metric(b)[0])
    eps = np.random.default_rng(seed).standard_normal((C, ot.dim))
    return b + np.linalg.solve(L.T, eps.T).T
