"""Iterative NUTS over the CUDA kernel, with the RMHMC, dense-LMC or
LMC-Monge dynamics.

Mirrors the reference's three NUTS samplers:

* ``nutsrmhmc(target, step_size, max_num_doublings=10,
  divergence_threshold=1000, integrator="implicit_midpoint",
  stopping_criterion="euc")`` (``rmhmc/nuts.py:164-250``);
* ``nutslmc(target, step_size, ...)`` (``lmcmc/nuts.py``, exported by the
  reference as ``nutslmc``);
* ``nutslmcmonge(target, step_size, inverse_mass_matrix, alpha2, ...)``
  (``lmcmonge/nuts.py``, exported as ``nutslmcmonge``).

Each returns ``SamplingAlgorithm(init, step)``; ``build_kernel()`` returns the
reference-shaped kernel.  Every chain builds its own trajectory (one thread
per chain, ``gj_nuts_step``), so chains whose trees stop early idle until the
deepest tree of their warp is done: the reference's ``vmap`` of a
``while_loop`` runs every chain for as long as the longest one too.

``rng_key`` is ``NUTSDraws(z, u)``, with z [C, d] momentum normals and u
[C, 2M + 2^M − 1] uniforms in the layout the C ABI documents, or an int seed
/ ``torch.Generator`` from which both are drawn on the device.
"""
from __future__ import annotations

import ctypes
from typing import Any, NamedTuple

import torch

from . import _lib as L
from .base import SamplingAlgorithm
from .samplers import INTEGRATORS, _init
from .targets import PRECISIONS, Target

CRITERIA = {"euc": 0, "bet": 1, "riem": 2}


class NUTSDraws(NamedTuple):
    z: Any  # [C, d] standard normals (the momentum draw)
    u: Any  # [C, 2M + 2^M − 1] uniforms (directions, merges, progressive samples)


class NUTSInfo(NamedTuple):
    """``rmhmc/nuts.py:37-75`` (the LMC samplers' info has the drawn
    velocity in the first field); the trajectory's extreme states are given
    by their positions."""

    momentum: Any
    is_divergent: Any
    is_turning: Any
    energy: Any
    trajectory_leftmost_position: Any
    trajectory_rightmost_position: Any
    num_trajectory_expansions: Any
    num_integration_steps: Any
    acceptance_rate: Any
    fixed_point_iters: Any
    status: Any


def num_uniforms(max_num_doublings: int) -> int:
    return 2 * max_num_doublings + 2 ** max_num_doublings - 1


class _Ctx:
    def __init__(self, target: Target, C: int, sampler: int):
        self.lib = L.lib()
        self.desc = target.descriptor()
        h = ctypes.c_void_p()
        L.check(self.lib.gj_create(ctypes.byref(self.desc), sampler,
                                   PRECISIONS[target.precision], C, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gj_destroy(self.h)
            self.h = None


class NUTSKernel:
    def __init__(self, sampler=L.GJ_SAMPLER_RMHMC, integrator="implicit_midpoint",
                 divergence_threshold=1000.0, max_iters=100, tol=1e-6, alpha2_fix=False):
        if integrator not in INTEGRATORS:
            raise ValueError(f"integrator must be one of {sorted(INTEGRATORS)}")
        self.sampler = sampler
        self.integrator = INTEGRATORS[integrator]
        self.divergence_threshold = float(divergence_threshold)
        self.max_iters = int(max_iters)
        self.tol = float(tol)
        self.alpha2_fix = bool(alpha2_fix)
        self._ctx = {}

    def _context(self, target, C):
        key = (id(target), C)
        if key not in self._ctx:
            self._ctx[key] = _Ctx(target, C, self.sampler)
        return self._ctx[key]

    @staticmethod
    def draws(key, C, d, M, target):
        U = num_uniforms(M)
        if isinstance(key, NUTSDraws):
            z = torch.as_tensor(key.z).to(device=target.device, dtype=target.dtype).contiguous()
            u = torch.as_tensor(key.u).to(device=target.device, dtype=torch.float64).contiguous()
        else:
            gen = key if isinstance(key, torch.Generator) else torch.Generator(device=target.device)
            if not isinstance(key, torch.Generator):
                gen.manual_seed(int(key))
            z = torch.randn(C, d, generator=gen, device=target.device, dtype=target.dtype)
            u = torch.rand(C, U, generator=gen, device=target.device, dtype=torch.float64)
        if z.shape != (C, d) or u.ndim != 2 or u.shape[0] != C or u.shape[1] < U:
            raise ValueError(f"draws must be z[{C}, {d}] and u[{C}, >= {U}]")
        return z, u

    def __call__(self, rng_key, state, target, step_size, max_num_doublings=10,
                 stopping_criterion="euc", *, alpha2=0.0, inverse_mass_matrix=None):
        if stopping_criterion not in CRITERIA:
            raise ValueError(f"stopping_criterion must be one of {sorted(CRITERIA)}")
        C, d = state.position.shape
        M = int(max_num_doublings)
        z, u = self.draws(rng_key, C, d, M, target)
        ctx = self._context(target, C)
        new = type(state)(*(t.clone() for t in state))
        im = None
        if inverse_mass_matrix is not None:
            im = torch.as_tensor(inverse_mass_matrix).to(device=target.device,
                                                         dtype=target.dtype).contiguous()
        dev, dt = target.device, target.dtype
        info = {
            "acceptance_rate": torch.empty(C, dtype=torch.float64, device=dev),
            "is_divergent": torch.empty(C, dtype=torch.uint8, device=dev),
            "is_turning": torch.empty(C, dtype=torch.uint8, device=dev),
            "energy": torch.empty(C, dtype=torch.float64, device=dev),
            "num_trajectory_expansions": torch.empty(C, dtype=torch.int32, device=dev),
            "num_integration_steps": torch.empty(C, dtype=torch.int32, device=dev),
            "fp_iters": torch.empty(C, dtype=torch.int32, device=dev),
            "status": torch.empty(C, dtype=torch.uint8, device=dev),
            "momentum": torch.empty(C, d, dtype=dt, device=dev),
            "leftmost_position": torch.empty(C, d, dtype=dt, device=dev),
            "rightmost_position": torch.empty(C, d, dtype=dt, device=dev),
        }
        p = L.GjNutsParams(float(step_size), M, self.integrator, CRITERIA[stopping_criterion],
                           self.max_iters, self.tol, self.divergence_threshold, float(alpha2),
                           L.ptr(im), int(self.alpha2_fix), 0)
        st = L.GjChainState(L.ptr(new.position), L.ptr(new.logdensity_grad),
                            L.ptr(new.logdensity),
                            L.ptr(getattr(new, "volume_adjustment", None)), C)
        inf = L.GjNutsInfo(*(L.ptr(info[k]) for k in L.NUTS_INFO_FIELDS))
        L.check(ctx.lib.gj_nuts_step(ctx.h, ctypes.byref(p), ctypes.byref(st), L.ptr(z),
                                           L.ptr(u), u.shape[1], ctypes.byref(inf),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return new, NUTSInfo(info["momentum"], info["is_divergent"].bool(),
                             info["is_turning"].bool(), info["energy"], info["leftmost_position"],
                             info["rightmost_position"], info["num_trajectory_expansions"],
                             info["num_integration_steps"], info["acceptance_rate"],
                             info["fp_iters"], info["status"])


class nutsrmhmc:
    """Riemannian NUTS (``rmhmc/nuts.py:164-250``)."""

    @staticmethod
    def init(position, target: Target):
        return _init(target, position, False)

    @staticmethod
    def build_kernel(integrator="implicit_midpoint", divergence_threshold=1000.0, max_iters=100,
                     tol=1e-6):
        return NUTSKernel(L.GJ_SAMPLER_RMHMC, integrator, divergence_threshold, max_iters, tol)

    def __new__(cls, target: Target, step_size: float, *, max_num_doublings: int = 10,
                divergence_threshold=1000.0, integrator="implicit_midpoint",
                stopping_criterion: str = "euc", max_iters=100, tol=1e-6):
        kernel = cls.build_kernel(integrator, divergence_threshold, max_iters, tol)

        def init_fn(position):
            return cls.init(position, target)

        def step_fn(rng_key, state):
            return kernel(rng_key, state, target, step_size, max_num_doublings,
                          stopping_criterion=stopping_criterion)

        return SamplingAlgorithm(init_fn, step_fn)


class nutslmc:
    """NUTS with the dense-metric LMC dynamics (``lmcmc/nuts.py``)."""

    @staticmethod
    def init(position, target: Target):
        return _init(target, position, True)

    @staticmethod
    def build_kernel(divergence_threshold=1000.0):
        return NUTSKernel(L.GJ_SAMPLER_LMC, divergence_threshold=divergence_threshold)

    def __new__(cls, target: Target, step_size: float, *, max_num_doublings: int = 10,
                divergence_threshold=1000.0, stopping_criterion: str = "euc"):
        kernel = cls.build_kernel(divergence_threshold)

        def init_fn(position):
            return cls.init(position, target)

        def step_fn(rng_key, state):
            return kernel(rng_key, state, target, step_size, max_num_doublings,
                          stopping_criterion=stopping_criterion)

        return SamplingAlgorithm(init_fn, step_fn)


class nutslmcmonge:
    """NUTS with the LMC-Monge dynamics (``lmcmonge/nuts.py``, the reference's
    ``nutslmc`` of that module); ``kernel(rng_key, state, target, step_size,
    inverse_mass_matrix, alpha2, stopping_criterion="euc")`` with
    ``max_num_doublings`` given to ``build_kernel`` as there."""

    @staticmethod
    def init(position, target: Target):
        return _init(target, position, True)

    @staticmethod
    def build_kernel(divergence_threshold=1000.0, max_num_doublings: int = 10, alpha2_fix=False):
        base = NUTSKernel(L.GJ_SAMPLER_LMCMONGE, divergence_threshold=divergence_threshold,
                          alpha2_fix=alpha2_fix)

        def kernel(rng_key, state, target, step_size, inverse_mass_matrix, alpha2,
                   stopping_criterion="euc"):
            return base(rng_key, state, target, step_size, max_num_doublings, stopping_criterion,
                        alpha2=alpha2, inverse_mass_matrix=inverse_mass_matrix)

        return kernel

    def __new__(cls, target: Target, step_size: float, inverse_mass_matrix, *, alpha2=0.001,
                max_num_doublings: int = 10, divergence_threshold=1000.0,
                stopping_criterion: str = "euc", alpha2_fix=False):
        kernel = cls.build_kernel(divergence_threshold, max_num_doublings, alpha2_fix)

        def init_fn(position):
            return cls.init(position, target)

        def step_fn(rng_key, state):
            return kernel(rng_key, state, target, step_size, inverse_mass_matrix, alpha2,
                          stopping_criterion)

        return SamplingAlgorithm(init_fn, step_fn)
