"""geomjax-shaped sampler API over the CUDA kernels.

Mirrors the reference's user interface:

* ``rmhmc(target, step_size, num_integration_steps, ...)`` ↔
  ``geomjax.rmhmc(logdensity_fn, step_size, metric_fn, num_integration_steps,
  divergence_threshold=1000, integrator=implicit_midpoint)``
  (``rmhmc/rmhmc.py:247-311``);
* ``lmcmonge(target, step_size, inverse_mass_matrix, num_integration_steps,
  alpha2=0.001)`` ↔ ``geomjax.lmcmonge`` (``lmcmonge/lmc.py:312-405``);
* ``lmc(target, step_size, num_integration_steps)`` ↔ ``geomjax.lmc``
  (``lmcmc/lmc.py:255-330``).

Each returns ``SamplingAlgorithm(init, step)``; ``build_kernel()`` returns
the reference-shaped ``kernel(rng_key, state, target, step_size, ...)``.
The target's registered metric plays the role of ``metric_fn``.
``rng_key`` is either ``Draws(z, u)`` (explicit randomness, as the oracle
uses) or an int seed / ``torch.Generator`` from which z ~ N(0, 1) and
u ~ U(0, 1) are drawn on the device.  Steps are pure: the input state is
not modified.  ``Kernel.step_inplace`` is the allocation-free variant used
in long loops.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib as L
from .base import (Draws, LMCInfo, LMCState, Proposal, RMHMCInfo, RMHMCState, SamplingAlgorithm)
from .targets import PRECISIONS, Target

INTEGRATORS = {"implicit_midpoint": L.GJ_IMPLICIT_MIDPOINT,
               "generalized_leapfrog": L.GJ_GENERALIZED_LEAPFROG}
LOGREG_PATHS = {"auto": 0, "simt": 1, "tcgen05": 2, "per_chain": 3, "cta": 4}


def cta_supported(N: int, d: int, precision: str = "fp64", lmc: bool = False) -> bool:
    """Whether one chain of an N x d logistic regression fits the
    CTA-per-chain kernels (d <= 64 and the shared-memory layout of
    csrc/logreg_cta.cu within 227 KB; the header gives the same formula)."""
    if d < 1 or d > 64 or N < 1:
        return False
    P = d * (d + 1) // 2
    t = 4 if precision == "mixed" else 8
    nd = 2 * P + 16 * d + 274 + ((P + d * d) if lmc else 0)
    b = nd * 8 + (P * 4 if t == 4 else 0) + (4 * N + max(N, 16 * d)) * t
    b = (b + 15) // 16 * 16 + 16 * (d + 1) * t
    b = (b + 15) // 16 * 16 + (4 * d if lmc else 0)
    return (b + 15) // 16 * 16 <= 227 * 1024


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Context:
    """Owns one gj_ctx (target x sampler x precision x chain count)."""

    def __init__(self, target: Target, sampler: int, C: int, options: dict):
        lib = L.lib()
        self.lib = lib
        self.target = target
        self.desc = target.descriptor()
        h = ctypes.c_void_p()
        L.check(lib.gj_create(ctypes.byref(self.desc), sampler, PRECISIONS[target.precision], C,
                              ctypes.byref(h)))
        self.h = h
        self.C = C
        for k, v in options.items():
            L.check(lib.gj_set_option(self.h, k, int(v)))

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gj_destroy(self.h)
            self.h = None


class Kernel:
    """A reference-shaped transition kernel bound to one sampler kind."""

    def __init__(self, sampler: int, integrator="implicit_midpoint", divergence_threshold=1000.0,
                 max_iters=100, tol=1e-6, alpha2_fix=False, logreg_path="auto", threads_per_block=None,
                 loop="graph", cholesky="fp64", chol_chains_per_warp=0, chain_groups=0,
                 pdl=False, gemm_ksplit=0, fuse_r2x=True, refine_iterates=True):
        if integrator not in INTEGRATORS:
            raise ValueError(f"integrator must be one of {sorted(INTEGRATORS)}")
        if logreg_path not in LOGREG_PATHS:
            raise ValueError(f"logreg_path must be one of {sorted(LOGREG_PATHS)}")
        self.sampler = sampler
        self.integrator = INTEGRATORS[integrator]
        self.divergence_threshold = float(divergence_threshold)
        self.max_iters = int(max_iters)
        self.tol = float(tol)
        self.alpha2_fix = bool(alpha2_fix)
        if loop not in ("graph", "host"):
            raise ValueError("loop must be 'graph' or 'host'")
        if cholesky not in ("fp64", "fp32"):
            raise ValueError("cholesky must be 'fp64' or 'fp32'")
        self.options = {L.GJ_OPT_LOGREG_PATH: LOGREG_PATHS[logreg_path],
                        L.GJ_OPT_LOOP: 0 if loop == "graph" else 1,
                        L.GJ_OPT_CHOL_FP64: 1 if cholesky == "fp64" else 0}
        if chol_chains_per_warp:
            self.options[L.GJ_OPT_CHOL_CHAINS_PER_WARP] = int(chol_chains_per_warp)
        if chain_groups:
            self.options[L.GJ_OPT_CHAIN_GROUPS] = int(chain_groups)
        self.options[L.GJ_OPT_PDL] = 1 if pdl else 0
        if gemm_ksplit:
            self.options[L.GJ_OPT_GEMM_KSPLIT] = int(gemm_ksplit)
        self.options[L.GJ_OPT_FUSE_R2X] = 1 if fuse_r2x else 0
        self.options[L.GJ_OPT_REFINE_ITERATES] = 1 if refine_iterates else 0
        if threads_per_block:
            self.options[L.GJ_OPT_THREADS_PER_BLOCK] = int(threads_per_block)
        self._ctx = {}

    def context(self, target: Target, C: int) -> _Context:
        key = (id(target), C)
        c = self._ctx.get(key)
        if c is None:
            c = _Context(target, self.sampler, C, self.options)
            self._ctx[key] = c
        return c

    def params(self, target, step_size, num_integration_steps, alpha2=0.0, inverse_mass=None):
        p = L.GjStepParams()
        p.step_size = float(step_size)
        p.num_integration_steps = int(num_integration_steps)
        p.integrator = self.integrator
        p.max_iters = self.max_iters
        p.tol = self.tol
        p.divergence_threshold = self.divergence_threshold
        p.alpha2 = float(alpha2)
        p.inverse_mass = L.ptr(inverse_mass)
        p.alpha2_fix = int(self.alpha2_fix)
        p.reserved = 0
        return p

    # -- randomness --------------------------------------------------------
    @staticmethod
    def draws(key, C, d, target: Target):
        if isinstance(key, Draws):
            z = torch.as_tensor(key.z).to(device=target.device, dtype=target.dtype).contiguous()
            u = torch.as_tensor(key.u).to(device=target.device, dtype=torch.float64).contiguous()
        else:
            if isinstance(key, torch.Generator):
                gen = key
            else:
                gen = torch.Generator(device=target.device)
                gen.manual_seed(int(key))
            z = torch.randn(C, d, generator=gen, device=target.device, dtype=target.dtype)
            u = torch.rand(C, generator=gen, device=target.device, dtype=torch.float64)
        if z.shape != (C, d) or u.shape != (C,):
            raise ValueError(f"draws must be z[{C}, {d}] and u[{C}]")
        return z, u

    # -- one transition ----------------------------------------------------
    def step_inplace(self, target, state, z, u, info, step_size, num_integration_steps, *,
                     alpha2=0.0, inverse_mass=None):
        """Advance ``state`` (modified in place) by one transition; ``info`` is
        a dict of preallocated device tensors (or None entries)."""
        C = state.position.shape[0]
        ctx = self.context(target, C)
        st = L.GjChainState(L.ptr(state.position), L.ptr(state.logdensity_grad),
                            L.ptr(state.logdensity),
                            L.ptr(getattr(state, "volume_adjustment", None)), C)
        inf = L.GjInfo(*(L.ptr(info.get(k)) for k in L.INFO_FIELDS))
        p = self.params(target, step_size, num_integration_steps, alpha2, inverse_mass)
        fn = {L.GJ_SAMPLER_RMHMC: ctx.lib.gj_rmhmc_step, L.GJ_SAMPLER_LMC: ctx.lib.gj_lmc_step,
              L.GJ_SAMPLER_LMCMONGE: ctx.lib.gj_lmcmonge_step}[self.sampler]
        L.check(fn(ctx.h, ctypes.byref(p), ctypes.byref(st), L.ptr(z), L.ptr(u), ctypes.byref(inf),
                   _stream()))

    @staticmethod
    def new_info(C, d, target, device, proposal=False):
        """Output buffers of one transition; with ``proposal`` also the
        flipped end state (``proposal_position``, ``proposal_velocity``)."""
        info = {
            "acceptance_rate": torch.empty(C, dtype=torch.float64, device=device),
            "is_accepted": torch.empty(C, dtype=torch.uint8, device=device),
            "is_divergent": torch.empty(C, dtype=torch.uint8, device=device),
            "energy": torch.empty(C, dtype=torch.float64, device=device),
            "fp_iters": torch.empty(C, dtype=torch.int32, device=device),
            "status": torch.empty(C, dtype=torch.uint8, device=device),
            "momentum": torch.empty(C, d, dtype=target.dtype, device=device),
        }
        if proposal:
            info["proposal_position"] = torch.empty(C, d, dtype=target.dtype, device=device)
            info["proposal_velocity"] = torch.empty(C, d, dtype=target.dtype, device=device)
        return info

    def __call__(self, rng_key, state, target, step_size, num_integration_steps, *, alpha2=0.0,
                 inverse_mass_matrix=None):
        C, d = state.position.shape
        z, u = self.draws(rng_key, C, d, target)
        new = type(state)(*(t.clone() for t in state))
        info = self.new_info(C, d, target, target.device, proposal=True)
        im = None
        if inverse_mass_matrix is not None:
            im = torch.as_tensor(inverse_mass_matrix).to(device=target.device, dtype=target.dtype)
            im = im.contiguous()
        self.step_inplace(target, new, z, u, info, step_size, num_integration_steps, alpha2=alpha2,
                          inverse_mass=im)
        acc = info["is_accepted"].bool()
        div = info["is_divergent"].bool()
        prop = Proposal(info["proposal_position"], info["proposal_velocity"])
        if self.sampler == L.GJ_SAMPLER_RMHMC:
            return new, RMHMCInfo(info["momentum"], info["acceptance_rate"], acc, div,
                                  info["energy"], num_integration_steps, info["fp_iters"],
                                  info["status"], prop)
        return new, LMCInfo(info["momentum"], info["acceptance_rate"], acc, div, info["energy"],
                            num_integration_steps, info["status"], prop)


def _init(target: Target, position, lmc_state: bool):
    lib = L.lib()
    q = torch.as_tensor(position).to(device=target.device, dtype=target.dtype).contiguous()
    if q.ndim == 1:
        q = q[None]
    if q.ndim != 2 or q.shape[1] != target.dim:
        raise ValueError(f"positions must be [chains, {target.dim}]")
    C = q.shape[0]
    ld = torch.empty(C, dtype=torch.float64, device=target.device)
    g = torch.empty_like(q)
    desc = target.descriptor()
    L.check(lib.gj_logdensity_grad(ctypes.byref(desc), PRECISIONS[target.precision], C, L.ptr(q),
                                   L.ptr(ld), L.ptr(g), _stream()))
    if lmc_state:
        return LMCState(q, ld, g, torch.zeros(C, dtype=torch.float64, device=target.device))
    return RMHMCState(q, ld, g)


class rmhmc:
    """Riemannian manifold HMC (``rmhmc/rmhmc.py:247-311``)."""

    @staticmethod
    def init(position, target: Target):
        """``rmhmc.py:96-98``."""
        return _init(target, position, False)

    @staticmethod
    def build_kernel(integrator="implicit_midpoint", divergence_threshold=1000.0, max_iters=100,
                     tol=1e-6, logreg_path="auto", loop="graph", cholesky="fp64",
                     chol_chains_per_warp=0, chain_groups=0, pdl=False, gemm_ksplit=0,
                     fuse_r2x=True, refine_iterates=True):
        """``rmhmc.py:110-176``; kernel(rng_key, state, target, step_size,
        num_integration_steps).  ``logreg_path``, ``loop``, ``cholesky``,
        ``chol_chains_per_warp``, ``chain_groups``, ``pdl``, ``gemm_ksplit``
        (K slices of the gradient contraction, 0 = automatic), ``fuse_r2x``
        (the momentum evaluations' r₂·X inside the S GEMM's epilogue) and
        ``refine_iterates`` (the generalized leapfrog's position-iterate
        solves by an FP32 factorisation refined with FP64 residuals) select
        the implementation of the batched dense-Fisher path."""
        return Kernel(L.GJ_SAMPLER_RMHMC, integrator, divergence_threshold, max_iters, tol,
                      logreg_path=logreg_path, loop=loop, cholesky=cholesky,
                      chol_chains_per_warp=chol_chains_per_warp, chain_groups=chain_groups,
                      pdl=pdl, gemm_ksplit=gemm_ksplit, fuse_r2x=fuse_r2x,
                      refine_iterates=refine_iterates)

    def __new__(cls, target: Target, step_size: float, num_integration_steps: int, *,
                divergence_threshold=1000.0, integrator="implicit_midpoint", max_iters=100,
                tol=1e-6, logreg_path="auto"):
        kernel = cls.build_kernel(integrator, divergence_threshold, max_iters, tol, logreg_path)

        def init_fn(position):
            return cls.init(position, target)

        def step_fn(rng_key, state):
            return kernel(rng_key, state, target, step_size, num_integration_steps)

        alg = SamplingAlgorithm(init_fn, step_fn)
        return alg


class lmcmonge:
    """LMC on a Monge patch (``lmcmonge/lmc.py:312-405``)."""

    @staticmethod
    def init(position, target: Target):
        """``lmcmonge/lmc.py:101-109``."""
        return _init(target, position, True)

    @staticmethod
    def build_kernel(divergence_threshold=1000.0, alpha2_fix=False, warp=True):
        """``lmcmonge/lmc.py:130-237``; kernel(rng_key, state, target,
        step_size, num_integration_steps, alpha2=..., inverse_mass_matrix=...).
        ``warp``: one warp per chain (default, either precision) or one thread
        per chain."""
        k = Kernel(L.GJ_SAMPLER_LMCMONGE, divergence_threshold=divergence_threshold,
                   alpha2_fix=alpha2_fix)
        k.options[L.GJ_OPT_MONGE_WARP] = 1 if warp else 0
        return k

    def __new__(cls, target: Target, step_size: float, inverse_mass_matrix, num_integration_steps:
                int, *, alpha2: float = 0.001, divergence_threshold=1000.0, alpha2_fix=False):
        kernel = cls.build_kernel(divergence_threshold, alpha2_fix)
        im = torch.as_tensor(inverse_mass_matrix).to(device=target.device, dtype=target.dtype)

        def init_fn(position):
            return cls.init(position, target)

        def step_fn(rng_key, state):
            return kernel(rng_key, state, target, step_size, num_integration_steps, alpha2=alpha2,
                          inverse_mass_matrix=im)

        return SamplingAlgorithm(init_fn, step_fn)


class lmc:
    """Lagrangian Monte Carlo with a dense position-dependent metric
    (``lmcmc/lmc.py:255-330``)."""

    @staticmethod
    def init(position, target: Target):
        """``lmcmc/lmc.py:98-101``."""
        return _init(target, position, True)

    @staticmethod
    def build_kernel(divergence_threshold=1000.0, logreg_path="auto"):
        """``lmcmc/lmc.py:114-182``.  ``logreg_path``: for the dense-Fisher
        logistic regression, "per_chain" runs one thread per chain (d <= 32);
        any other value one CTA per chain (d <= 64)."""
        return Kernel(L.GJ_SAMPLER_LMC, divergence_threshold=divergence_threshold,
                      logreg_path=logreg_path)

    def __new__(cls, target: Target, step_size: float, num_integration_steps: int, *,
                divergence_threshold=1000.0):
        kernel = cls.build_kernel(divergence_threshold)

        def init_fn(position):
            return cls.init(position, target)

        def step_fn(rng_key, state):
            return kernel(rng_key, state, target, step_size, num_integration_steps)

        return SamplingAlgorithm(init_fn, step_fn)
