"""Batches of independent dense-Fisher logistic-regression posteriors.

The reference samples one posterior per ``kernel`` call; a user with many
posteriors writes a loop (or a ``vmap`` over equally shaped ones) around
``geomjax.rmhmc`` (``rmhmc/rmhmc.py:131-174``).  ``PosteriorBatch`` is that
loop as one call: posteriors of different sizes (N and d may differ,
d <= 128), C chains each, one CUDA graph per posterior spread over a pool
of streams (``gj_batch_rmhmc_step``).

State layout (device tensors):

* ``position`` / ``logdensity_grad``: float32, ragged concatenation of the
  posteriors' [C, d_b] blocks (``offsets[b]`` is the start of block b);
* ``logdensity``: float64 [B*C].

``positions(state, b)`` returns posterior b's [C, d_b] view.

The graphs overlap only as far as the device's hardware work queues allow:
importing ``geomjax_gb300`` before CUDA starts sets
``CUDA_DEVICE_MAX_CONNECTIONS=32`` unless the environment sets it.
"""
from __future__ import annotations

import ctypes
from typing import NamedTuple, Sequence

import numpy as np
import torch

from . import _lib as L
from .base import Draws, RMHMCState
from .targets import logistic_regression


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class BatchInfo(NamedTuple):
    acceptance_rate: torch.Tensor  # [B*C] float64
    is_accepted: torch.Tensor      # [B*C] bool
    is_divergent: torch.Tensor     # [B*C] bool
    energy: torch.Tensor           # [B*C] float64
    fixed_point_iters: torch.Tensor  # [B*C] int32
    status: torch.Tensor           # [B*C] uint8
    momentum: torch.Tensor         # ragged float32


class PosteriorBatch:
    """B logistic-regression posteriors ``datasets = [(X_b, y_b), ...]``,
    ``chains`` RMHMC chains each (mixed precision; ``integrator``
    "implicit_midpoint", the reference's, or "generalized_leapfrog")."""

    def __init__(self, datasets: Sequence, chains: int, prior_var: float = 100.0,
                 num_streams: int = 16, max_iters: int = 100, tol: float = 1e-6,
                 divergence_threshold: float = 1000.0, device="cuda",
                 integrator: str = "implicit_midpoint", one_graph: bool = True,
                 grouped: bool = True, buckets: int = 0):
        self.lib = L.lib()
        self.device = torch.device(device)
        self.targets = [logistic_regression(X, y, prior_var=prior_var, precision="mixed",
                                            device=self.device) for X, y in datasets]
        self.B = len(self.targets)
        self.C = int(chains)
        self.dims = [t.dim for t in self.targets]
        self.offsets = np.concatenate([[0], np.cumsum([self.C * d for d in self.dims])])
        self.max_iters, self.tol = int(max_iters), float(tol)
        self.integrator = {"implicit_midpoint": L.GJ_IMPLICIT_MIDPOINT,
                           "generalized_leapfrog": L.GJ_GENERALIZED_LEAPFROG}[integrator]
        self.divergence_threshold = float(divergence_threshold)
        descs = (L.GjTarget * self.B)(*(t.descriptor() for t in self.targets))
        self._descs = descs
        h = ctypes.c_void_p()
        L.check(self.lib.gj_batch_create(ctypes.cast(descs, ctypes.c_void_p), self.B, self.C,
                                         int(num_streams), ctypes.byref(h)))
        self.h = h
        # one CUDA graph for the whole batch (with ``grouped``, the default,
        # every stage one grid over a bucket of posteriors, each bucket a
        # branch; otherwise every posterior a branch), or one graph per
        # posterior on the stream pool
        self.set_option(L.GJ_OPT_BATCH_GRAPH, (2 if grouped else 1) if one_graph else 0)
        if buckets:
            self.set_option(L.GJ_OPT_BATCH_BUCKETS, int(buckets))

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.gj_batch_destroy(self.h)
            self.h = None

    def set_option(self, key: int, value: int):
        L.check(self.lib.gj_batch_set_option(self.h, key, int(value)))

    # -- layout helpers ----------------------------------------------------
    def positions(self, state, b: int) -> torch.Tensor:
        o0, o1 = int(self.offsets[b]), int(self.offsets[b + 1])
        return state.position[o0:o1].view(self.C, self.dims[b])

    def pack(self, blocks: Sequence, dtype=torch.float32) -> torch.Tensor:
        """Concatenate per-posterior [C, d_b] arrays into the ragged layout."""
        parts = [torch.as_tensor(np.asarray(x), dtype=dtype).reshape(-1) for x in blocks]
        return torch.cat(parts).to(self.device).contiguous()

    # -- API -----------------------------------------------------------------
    def init(self, positions: Sequence) -> RMHMCState:
        """``rmhmc.py:96-98`` for every posterior; positions[b] is [C, d_b]."""
        q = self.pack(positions)
        g = torch.empty_like(q)
        ld = torch.empty(self.B * self.C, dtype=torch.float64, device=self.device)
        for b, t in enumerate(self.targets):
            qb = q[int(self.offsets[b]):int(self.offsets[b + 1])].view(self.C, t.dim)
            lb, gb = t.logdensity_and_grad(qb)
            ld[b * self.C:(b + 1) * self.C] = lb
            g[int(self.offsets[b]):int(self.offsets[b + 1])] = gb.reshape(-1)
        return RMHMCState(q, ld, g)

    def draws(self, key):
        n = int(self.offsets[-1])
        if isinstance(key, Draws):
            z = torch.as_tensor(key.z).to(device=self.device, dtype=torch.float32).reshape(-1)
            u = torch.as_tensor(key.u).to(device=self.device, dtype=torch.float64).reshape(-1)
            z, u = z.contiguous(), u.contiguous()
        else:
            gen = key if isinstance(key, torch.Generator) else torch.Generator(device=self.device)
            if not isinstance(key, torch.Generator):
                gen.manual_seed(int(key))
            z = torch.randn(n, generator=gen, device=self.device, dtype=torch.float32)
            u = torch.rand(self.B * self.C, generator=gen, device=self.device, dtype=torch.float64)
        if z.numel() != n or u.numel() != self.B * self.C:
            raise ValueError(f"draws must be z[{n}] (ragged) and u[{self.B * self.C}]")
        return z, u

    def new_info(self):
        n, BC = int(self.offsets[-1]), self.B * self.C
        dev = self.device
        return {"acceptance_rate": torch.empty(BC, dtype=torch.float64, device=dev),
                "is_accepted": torch.empty(BC, dtype=torch.uint8, device=dev),
                "is_divergent": torch.empty(BC, dtype=torch.uint8, device=dev),
                "energy": torch.empty(BC, dtype=torch.float64, device=dev),
                "fp_iters": torch.empty(BC, dtype=torch.int32, device=dev),
                "status": torch.empty(BC, dtype=torch.uint8, device=dev),
                "momentum": torch.empty(n, dtype=torch.float32, device=dev)}

    def step_inplace(self, state, z, u, info, step_size, num_integration_steps):
        p = L.GjStepParams()
        p.step_size = float(step_size)
        p.num_integration_steps = int(num_integration_steps)
        p.integrator = self.integrator
        p.max_iters = self.max_iters
        p.tol = self.tol
        p.divergence_threshold = self.divergence_threshold
        st = L.GjChainState(L.ptr(state.position), L.ptr(state.logdensity_grad),
                            L.ptr(state.logdensity), None, self.B * self.C)
        inf = L.GjInfo(*(L.ptr(info.get(k)) for k in L.INFO_FIELDS))
        L.check(self.lib.gj_batch_rmhmc_step(self.h, ctypes.byref(p), ctypes.byref(st), L.ptr(z),
                                             L.ptr(u), ctypes.byref(inf), _stream()))

    def step(self, rng_key, state, step_size, num_integration_steps):
        """One transition of every chain of every posterior (pure: returns a
        new state)."""
        z, u = self.draws(rng_key)
        new = RMHMCState(*(t.clone() for t in state))
        info = self.new_info()
        self.step_inplace(new, z, u, info, step_size, num_integration_steps)
        return new, BatchInfo(info["acceptance_rate"], info["is_accepted"].bool(),
                              info["is_divergent"].bool(), info["energy"], info["fp_iters"],
                              info["status"], info["momentum"])
