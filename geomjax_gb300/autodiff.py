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


class _TransitionStats(torch.autograd.Function):
    """Mean acceptance probability and mean energy error of one generalized-
    leapfrog RMHMC transition as differentiable functions of the step size h
    and the metric regulariser λ (logistic regression, float64).  The forward
    pass runs the tangent kernel once and keeps the 2 x 2 Jacobian of the two
    means; the backward pass is that Jacobian's transpose times the incoming
    gradients (exact for the discrete trajectory with fixed iteration
    counts)."""

    @staticmethod
    def forward(ctx, h, lam, target, q0, z, nsteps, kp, kq):
        out = transition_jacobian(target, q0, z, float(h), float(lam), nsteps, kp, kq)
        ctx.jac = out.mean(dim=0)  # (p, dp/dh, dp/dλ, ΔH, dΔH/dh, dΔH/dλ)
        return ctx.jac[0].clone(), ctx.jac[3].clone()

    @staticmethod
    def backward(ctx, gp, gdh):
        j = ctx.jac
        gh = gp * j[1] + gdh * j[4]
        gl = gp * j[2] + gdh * j[5]
        return gh, gl, None, None, None, None, None, None


def transition_stats(target, q0, z, step_size, metric_reg, num_integration_steps, kp=6, kq=6):
    """(mean p_accept, mean ΔH) of one generalized-leapfrog transition from
    positions q0 with momentum normals z; differentiable in ``step_size`` and
    ``metric_reg`` (0-d float64 tensors with requires_grad)."""
    if target.precision != "fp64" or target.family != L.GJ_LOGREG:
        raise ValueError("transition_stats needs a float64 logistic-regression target")
    q0 = torch.as_tensor(q0, dtype=torch.float64).to(target.device).contiguous()
    z = torch.as_tensor(z, dtype=torch.float64).to(target.device).contiguous()
    return _TransitionStats.apply(step_size, metric_reg, target, q0, z, num_integration_steps, kp, kq)


def transition_values(target, q0, z, step_size, metric_reg, num_integration_steps, kp=6, kq=6):
    """Per-chain (p_accept, ΔH) without tangents (used for finite differences)."""
    lib = L.lib()
    q0 = torch.as_tensor(q0, dtype=torch.float64).to(target.device).contiguous()
    z = torch.as_tensor(z, dtype=torch.float64).to(target.device).contiguous()
    out = torch.empty(q0.shape[0], 6, dtype=torch.float64, device=target.device)
    d = target.descriptor()
    L.check(lib.gj_logreg_gl_transition_jvp(ctypes.byref(d), q0.shape[0], L.ptr(q0), L.ptr(z),
                                            float(step_size), float(metric_reg),
                                            int(num_integration_steps), int(kp), int(kq), 0,
                                            L.ptr(out), _stream()))
    return out[:, 0], out[:, 3]


def transition_jacobian(target, q0, z, step_size, metric_reg, num_integration_steps, kp=6, kq=6):
    """Per-chain [C, 6] output of the tangent kernel."""
    lib = L.lib()
    q0 = torch.as_tensor(q0, dtype=torch.float64).to(target.device).contiguous()
    z = torch.as_tensor(z, dtype=torch.float64).to(target.device).contiguous()
    out = torch.empty(q0.shape[0], 6, dtype=torch.float64, device=target.device)
    d = target.descriptor()
    L.check(lib.gj_logreg_gl_transition_jvp(ctypes.byref(d), q0.shape[0], L.ptr(q0), L.ptr(z),
                                            float(step_size), float(metric_reg),
                                            int(num_integration_steps), int(kp), int(kq), 1,
                                            L.ptr(out), _stream()))
    return out


def lmcmonge_alpha2_tangent(target: Target, positions, z, step_size: float,
                            num_integration_steps: int, alpha2: float, inverse_mass_matrix=None,
                            alpha2_fix: bool = False):
    """Proposal position q_L of one LMC-Monge transition from ``positions``
    with normals ``z``, and ∂q_L/∂α² (``gj_lmcmonge_alpha2_jvp``, forward
    mode in float64 through the velocity draw and every half step).  The
    reference takes it with ``jax.jacfwd`` of the proposal position
    (``adaptation/chees_adaptation_lmcmonge.py:469-519``).  Returns two
    [C, d] tensors in the target's dtype."""
    q = _q(target, torch.as_tensor(positions))
    zz = torch.as_tensor(z).to(device=target.device, dtype=target.dtype).contiguous()
    if zz.shape != q.shape:
        raise ValueError("z must have the positions' shape")
    im = None
    if inverse_mass_matrix is not None:
        im = torch.as_tensor(inverse_mass_matrix).to(device=target.device,
                                                     dtype=target.dtype).contiguous()
    p = L.GjStepParams()
    p.step_size = float(step_size)
    p.num_integration_steps = int(num_integration_steps)
    p.integrator = 0
    p.max_iters = 0
    p.tol = 0.0
    p.divergence_threshold = 1000.0
    p.alpha2 = float(alpha2)
    p.inverse_mass = L.ptr(im)
    p.alpha2_fix = int(bool(alpha2_fix))
    p.reserved = 0
    qL = torch.empty_like(q)
    dq = torch.empty_like(q)
    desc = target.descriptor()
    L.check(L.lib().gj_lmcmonge_alpha2_jvp(ctypes.byref(desc), PRECISIONS[target.precision],
                                           q.shape[0], ctypes.byref(p), L.ptr(q), L.ptr(zz),
                                           L.ptr(qL), L.ptr(dq), _stream()))
    return qL, dq
