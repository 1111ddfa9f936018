"""Registered device target families.

The reference takes arbitrary Python callables ``logdensity_fn`` and
``metric_fn`` and differentiates them with JAX (``rmhmc/rmhmc.py:131-138``,
``lmcmc/lmc.py:135-143``).  Arbitrary Python cannot run inside a CUDA
kernel, so the drop-in boundary is a registry of families whose log density,
gradient, HVP and metric operators are written in CUDA
(``geomjax_gb300/csrc/targets.cuh``):

* ``funnel(D, sigma=3, metric="diag"|"pullback"|"identity")`` — Neal's funnel
  of ``examples/funnel/main.py:28-54`` (v = θ[D−1]);
* ``logistic_regression(X, y, prior_var=100, metric="fisher"|"identity")`` —
  Fisher metric XᵀΛX + I/prior_var;
* ``hierarchical_gaussian(y, sigma, mu_scale=5, v_scale=2)`` — arrowhead
  Fisher metric.

A target owns its data as device tensors of the precision's dtype
(float64 for ``"fp64"``, float32 for ``"mixed"``).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib as L

PRECISIONS = {"fp64": L.GJ_FP64, "mixed": L.GJ_MIXED}


def dtype_of(precision: str) -> torch.dtype:
    return torch.float64 if precision == "fp64" else torch.float32


class Target:
    family: int
    metric: int
    dim: int
    is_diagonal: bool

    def __init__(self, precision: str = "mixed", device="cuda"):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self.precision = precision
        self.dtype = dtype_of(precision)
        self.device = torch.device(device)
        self._keep = []

    def _tensor(self, x):
        t = torch.as_tensor(x, dtype=self.dtype).to(self.device).contiguous()
        self._keep.append(t)
        return t

    def descriptor(self) -> L.GjTarget:
        raise NotImplementedError

    # ---- operator-level calls (gj_logdensity_grad / gj_hvp / gj_metric) ----
    def _pos(self, q):
        q = torch.as_tensor(q).to(device=self.device, dtype=self.dtype).contiguous()
        if q.ndim != 2 or q.shape[1] != self.dim:
            raise ValueError(f"positions must be [chains, {self.dim}]")
        return q

    def logdensity_and_grad(self, q):
        lib = L.lib()
        q = self._pos(q)
        C = q.shape[0]
        ld = torch.empty(C, dtype=torch.float64, device=self.device)
        g = torch.empty_like(q)
        d = self.descriptor()
        L.check(lib.gj_logdensity_grad(ctypes.byref(d), PRECISIONS[self.precision], C, L.ptr(q),
                                       L.ptr(ld), L.ptr(g), _stream()))
        return ld, g

    def hvp(self, q, u):
        lib = L.lib()
        q = self._pos(q)
        u = self._pos(u)
        out = torch.empty_like(q)
        d = self.descriptor()
        L.check(lib.gj_hvp(ctypes.byref(d), PRECISIONS[self.precision], q.shape[0], L.ptr(q),
                           L.ptr(u), L.ptr(out), _stream()))
        return out

    def metric_fn(self, q):
        lib = L.lib()
        q = self._pos(q)
        C = q.shape[0]
        shape = (C, self.dim) if self.is_diagonal else (C, self.dim, self.dim)
        out = torch.empty(shape, dtype=self.dtype, device=self.device)
        d = self.descriptor()
        L.check(lib.gj_metric(ctypes.byref(d), PRECISIONS[self.precision], C, L.ptr(q), L.ptr(out),
                              _stream()))
        return out


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class funnel(Target):
    """Neal's funnel, v = θ[D−1] ~ N(0, σ²), θ[:D−1] | v ~ N(0, e^v)."""

    METRICS = {"diag": L.GJ_METRIC_DIAG_FISHER, "pullback": L.GJ_METRIC_PULLBACK,
               "identity": L.GJ_METRIC_IDENTITY}

    def __init__(self, D: int = 2, sigma: float = 3.0, metric: str = "diag", precision="mixed",
                 device="cuda"):
        super().__init__(precision, device)
        if metric not in self.METRICS:
            raise ValueError(f"funnel metric must be one of {sorted(self.METRICS)}")
        self.D = self.dim = int(D)
        self.sigma = float(sigma)
        self.metric_name = metric
        self.family = L.GJ_FUNNEL
        self.metric = self.METRICS[metric]
        self.is_diagonal = metric == "diag"

    def descriptor(self):
        return L.GjTarget(self.family, self.metric, self.dim, 0, None, None, None, self.sigma, 0.0)


class logistic_regression(Target):
    """Bayesian logistic regression with prior N(0, prior_var·I) and the
    Fisher metric G = XᵀΛ(β)X + I/prior_var."""

    METRICS = {"fisher": L.GJ_METRIC_DENSE_FISHER, "identity": L.GJ_METRIC_IDENTITY}

    def __init__(self, X, y, prior_var: float = 100.0, metric: str = "fisher", precision="mixed",
                 device="cuda"):
        super().__init__(precision, device)
        if metric not in self.METRICS:
            raise ValueError(f"logistic_regression metric must be one of {sorted(self.METRICS)}")
        self.X = self._tensor(X)
        self.y = self._tensor(y)
        if self.X.ndim != 2 or self.y.shape != (self.X.shape[0],):
            raise ValueError("X must be [N, d] and y [N]")
        self.N, self.dim = self.X.shape
        self.prior_var = float(prior_var)
        self.family = L.GJ_LOGREG
        self.metric_name = metric
        self.metric = self.METRICS[metric]
        self.is_diagonal = False

    def descriptor(self):
        return L.GjTarget(self.family, self.metric, self.dim, self.N, L.ptr(self.X), L.ptr(self.y),
                          None, self.prior_var, 0.0)


class hierarchical_gaussian(Target):
    """θ = [θ_1..θ_J, μ, v]; y_j ~ N(θ_j, σ_j²), θ_j ~ N(μ, e^v), μ ~ N(0, mu_scale²),
    v ~ N(0, v_scale²); arrowhead Fisher metric."""

    METRICS = {"fisher": L.GJ_METRIC_DENSE_FISHER, "identity": L.GJ_METRIC_IDENTITY}

    def __init__(self, y, sigma, mu_scale: float = 5.0, v_scale: float = 2.0, metric="fisher",
                 precision="mixed", device="cuda"):
        super().__init__(precision, device)
        self.y = self._tensor(y)
        self.sigma = self._tensor(sigma)
        self.J = int(self.y.shape[0])
        self.dim = self.J + 2
        self.mu_scale = float(mu_scale)
        self.v_scale = float(v_scale)
        self.family = L.GJ_HIERGAUSS
        self.metric_name = metric
        self.metric = self.METRICS[metric]
        self.is_diagonal = False

    def descriptor(self):
        return L.GjTarget(self.family, self.metric, self.dim, self.J, None, L.ptr(self.y),
                          L.ptr(self.sigma), self.mu_scale, self.v_scale)
