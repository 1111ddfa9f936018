"""torch.autograd bindings of the target operators with hand-written adjoints.

The reference obtains every derivative by JAX autodiff of the user's
``logdensity_fn`` / ``metric_fn`` (``rmhmc/integrators.py:111-114``,
``util.py:120-121``, ``lmcmc/metrics.py:165``).  Here each operator is a CUDA
kernel and its vector-Jacobian product is a CUDA kernel too:

* ``logdensity(target, q)``: forward ℓ(q); adjoint ḡ ↦ ḡ·∇ℓ(q)
  (``gj_logdensity_grad``);
* ``grad_logdensity(target, q)``: forward ∇ℓ(q); adjoint v ↦ H(q)v
  (``gj_hvp``; the Hessian is symmetric);
* ``metric(target, q)``: forward G(q); adjoint W ↦ Σ_ab W_ab ∂G_ab/∂q
  (``gj_metric_vjp``).

All run on the device with no CPU fallback.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib as L
from .targets import PRECISIONS, Target


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _q(target: Target, q):
    q = q.detach().to(device=target.device, dtype=target.dtype).contiguous()
    if q.ndim != 2 or q.shape[1] != target.dim:
        raise ValueError(f"positions must be [chains, {target.dim}]")
    return q


class _LogDensity(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q, target):
        ld, g = target.logdensity_and_grad(_q(target, q))
        ctx.save_for_backward(g)
        return ld.to(q.dtype)

    @staticmethod
    def backward(ctx, gld):
        (g,) = ctx.saved_tensors
        return gld[:, None].to(g.dtype) * g, None


class _Grad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q, target):
        qq = _q(target, q)
        _, g = target.logdensity_and_grad(qq)
        ctx.save_for_backward(qq)
        ctx.target = target
        return g.to(q.dtype)

    @staticmethod
    def backward(ctx, v):
        (qq,) = ctx.saved_tensors
        return ctx.target.hvp(qq, v.to(qq.dtype).contiguous()), None


class _Metric(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q, target):
        qq = _q(target, q)
        ctx.save_for_backward(qq)
        ctx.target = target
        return target.metric_fn(qq).to(q.dtype)

    @staticmethod
    def backward(ctx, W):
        (qq,) = ctx.saved_tensors
        t = ctx.target
        lib = L.lib()
        W = W.to(device=t.device, dtype=t.dtype).contiguous()
        out = torch.empty_like(qq)
        d = t.descriptor()
        L.check(lib.gj_metric_vjp(ctypes.byref(d), PRECISIONS[t.precision], qq.shape[0], L.ptr(qq),
                                  L.ptr(W), L.ptr(out), _stream()))
        return out, None


def logdensity(target: Target, q):
    return _LogDensity.apply(q, target)


def grad_logdensity(target: Target, q):
    return _Grad.apply(q, target)


def metric(target: Target, q):
    return _Metric.apply(q, target)
