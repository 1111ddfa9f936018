"""Autotuner of the batched dense-Fisher path's launch choices.

The batched path has three knobs whose best values depend on the shape
(chains, N, d) and on the device:

* the tcgen05 GEMM tile policy (``gj_set_gemm_tiling``): the output-tile
  width for N > 64 (automatic, 64 or 128) and whether the operand ring is cut
  back so that two CTAs share an SM (automatic, yes, no);
* the chains per warp of the FP64 metric factorisation
  (``GJ_OPT_CHOL_CHAINS_PER_WARP``: automatic, 1, 2, 4 or 8);
* the K slices of the gradient contraction (``GJ_OPT_GEMM_KSPLIT``:
  automatic, 1, 2 or 4), tried in a second stage with the best tile policy
  and chains per warp of the first;
* for the per-chain kernels, the threads per block (32, 64 or 128).

``autotune`` times a few transitions of every candidate on a copy of the
chains' state (CUDA events on the current stream, after one untimed
transition that also captures the candidate's graph) and leaves the fastest
one set: the tile policy process-wide, the factorisation and K-slice choices
on the kernel's (or batch's) contexts.  The candidates' results differ only
in the order of floating-point sums.
"""
from __future__ import annotations

import ctypes
import itertools
from typing import NamedTuple, Sequence

import torch

from . import _lib as L

TILINGS = ((0, -1), (64, -1), (128, -1), (0, 1), (0, 0))
CHOL_CPW = (0, 1, 2, 4, 8)
KSPLIT = (0, 1, 2, 4)


class AutotuneResult(NamedTuple):
    best: dict                 # the chosen settings
    ms_per_transition: float   # their time
    table: list                # (settings, ms per transition) for every candidate


def _set_tiling(bn, two):
    L.check(L.lib().gj_set_gemm_tiling(int(bn), int(two)))


def _time(step, transitions):
    step()  # capture and warm
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(transitions):
        step()
    e1.record(st)
    e1.synchronize()
    return e0.elapsed_time(e1) / transitions


def _candidates(tilings, cpws, ksplit0):
    return [{"gemm_tiling": t, "chol_chains_per_warp": c, "gemm_ksplit": ksplit0}
            for t, c in itertools.product(tilings, cpws)]


def _search(cands, ksplits, apply, measure):
    """The first stage over ``cands``, then the other K slices with its
    best settings; every candidate ends up in the table.  ``apply(c)`` puts
    candidate c in force, ``measure()`` times the settings in force (ms per
    transition)."""
    table = []
    for c in cands:
        apply(c)
        table.append((c, measure()))
    best = min(table, key=lambda x: x[1])[0]
    if "gemm_ksplit" in best:
        for k in ksplits[1:]:
            c = dict(best, gemm_ksplit=int(k))
            apply(c)
            table.append((c, measure()))
    best, ms = min(table, key=lambda x: x[1])
    apply(best)
    return AutotuneResult(best, ms, table)


def autotune(kernel, target, state, step_size: float, num_integration_steps: int, *,
             transitions: int = 3, tilings: Sequence = TILINGS, chol_chains_per_warp: Sequence = CHOL_CPW,
             gemm_ksplit: Sequence = KSPLIT, seed: int = 0) -> AutotuneResult:
    """Tune a ``Kernel`` (``geomjax_gb300.rmhmc.build_kernel()`` etc.) for
    ``target`` and the chain count of ``state``; ``state`` is not modified."""
    from .samplers import Kernel

    if not isinstance(kernel, Kernel):
        raise TypeError("kernel must be a geomjax_gb300 Kernel")
    C, d = state.position.shape
    ctx = kernel.context(target, C)
    work = type(state)(*(t.clone() for t in state))
    info = kernel.new_info(C, d, target, target.device)
    gen = torch.Generator(device=target.device)
    gen.manual_seed(int(seed))
    z, u = kernel.draws(gen, C, d, target)
    batched = (target.family == L.GJ_LOGREG and target.metric == L.GJ_METRIC_DENSE_FISHER and
               target.precision == "mixed" and kernel.sampler == L.GJ_SAMPLER_RMHMC and
               kernel.options.get(L.GJ_OPT_LOGREG_PATH, 0) != 3)
    ksplits = tuple(gemm_ksplit) or (0,)
    cands = _candidates(tilings, chol_chains_per_warp, ksplits[0]) if batched else \
        [{"threads_per_block": t} for t in (32, 64, 128)]

    def apply(c):
        if "gemm_tiling" in c:
            _set_tiling(*c["gemm_tiling"])
            for key, opt in (("chol_chains_per_warp", L.GJ_OPT_CHOL_CHAINS_PER_WARP),
                             ("gemm_ksplit", L.GJ_OPT_GEMM_KSPLIT)):
                kernel.options[opt] = c[key]
                L.check(ctx.lib.gj_set_option(ctx.h, opt, c[key]))
        else:
            kernel.options[L.GJ_OPT_THREADS_PER_BLOCK] = c["threads_per_block"]
            L.check(ctx.lib.gj_set_option(ctx.h, L.GJ_OPT_THREADS_PER_BLOCK, c["threads_per_block"]))

    def step():
        kernel.step_inplace(target, work, z, u, info, step_size, num_integration_steps)

    return _search(cands, ksplits, apply, lambda: _time(step, transitions))


def autotune_batch(batch, state, step_size: float, num_integration_steps: int, *,
                   transitions: int = 2, tilings: Sequence = TILINGS,
                   chol_chains_per_warp: Sequence = CHOL_CPW, gemm_ksplit: Sequence = KSPLIT,
                   seed: int = 0) -> AutotuneResult:
    """The same for a ``PosteriorBatch``: the tile policy, the
    factorisation's chains per warp and the gradient contraction's K slices
    of all its posteriors."""
    work = type(state)(*(t.clone() for t in state))
    info = batch.new_info()
    z, u = batch.draws(int(seed))

    def apply(c):
        _set_tiling(*c["gemm_tiling"])
        batch.set_option(L.GJ_OPT_CHOL_CHAINS_PER_WARP, c["chol_chains_per_warp"])
        batch.set_option(L.GJ_OPT_GEMM_KSPLIT, c["gemm_ksplit"])

    def step():
        batch.step_inplace(work, z, u, info, step_size, num_integration_steps)

    ksplits = tuple(gemm_ksplit) or (0,)
    return _search(_candidates(tilings, chol_chains_per_warp, ksplits[0]), ksplits, apply,
                   lambda: _time(step, transitions))
