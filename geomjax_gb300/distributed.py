"""Replicas over ranks: chains (and posteriors) are independent, so a
multi-GPU run gives each rank its own chains and needs no collective while
sampling.  Collectives appear only around the sampling phase:

* the wall time of a measured phase is the maximum over ranks;
* the min-ESS over all chains (the reference's ESS over all chains,
  ``diagnostics.py:78-209``) needs only two statistics of each rank's
  chains: the sum of their autocovariances ([samples, d], one all-reduce)
  and their means ([chains, d], one all-gather).  No trace leaves its rank.

The functions take an initialised ``torch.distributed`` process group (NCCL
on GPUs, gloo on CPU) and run on a single process without one.
"""
from __future__ import annotations

import torch

from .diagnostics import autocovariance_stats, effective_sample_size, ess_from_stats


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def shard(total: int, rank: int, world: int):
    """[start, stop) of rank's share of `total` units, sizes differing by at
    most one."""
    base, extra = divmod(int(total), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(x: float, device=None) -> float:
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_chains(trace: torch.Tensor, chain_axis: int = 1) -> torch.Tensor:
    """Concatenate every rank's trace along the chain axis (all ranks must
    hold the same number of samples; chain counts may differ)."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return trace
    x = torch.movedim(trace, chain_axis, 0).contiguous()
    n = torch.tensor([x.shape[0]], dtype=torch.int64, device=x.device)
    sizes = [torch.zeros_like(n) for _ in range(dist.get_world_size())]
    dist.all_gather(sizes, n)
    cmax = int(max(int(s.item()) for s in sizes))
    pad = torch.zeros((cmax,) + tuple(x.shape[1:]), dtype=x.dtype, device=x.device)
    pad[: x.shape[0]] = x
    parts = [torch.empty_like(pad) for _ in sizes]
    dist.all_gather(parts, pad)
    full = torch.cat([p[: int(s.item())] for p, s in zip(parts, sizes)], dim=0)
    return torch.movedim(full, 0, chain_axis)


def global_min_ess(trace: torch.Tensor, chain_axis: int = 1, sample_axis: int = 0) -> float:
    """min over dimensions of the ESS over all ranks' chains.  Each rank
    reduces its own trace to (Σ_c autocovariance_c, chain means); the sums
    are all-reduced and the means all-gathered (chain counts may differ), so
    the traffic is samples·d + chains·d doubles, not the traces."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(torch.min(effective_sample_size(trace, chain_axis=chain_axis,
                                                     sample_axis=sample_axis)).item())
    acov_sum, means = autocovariance_stats(trace, chain_axis, sample_axis)
    dist.all_reduce(acov_sum, op=dist.ReduceOp.SUM)
    all_means = gather_chains(means, chain_axis=0)
    return float(torch.min(ess_from_stats(acov_sum, all_means)).item())
