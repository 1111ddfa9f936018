"""MCMC diagnostics on device-resident traces (torch; runs on the GPU when
the trace is there).

``effective_sample_size`` restates ``diagnostics.py:78-209``: centred FFT
autocovariance padded to next_fast_len(2n), mean over chains, Geyer's
initial positive sequence then the initial monotone sequence, τ̂ floored at
1/log10(MN), ESS = MN/τ̂.  ``potential_scale_reduction`` restates
``diagnostics.py:25-75``.
"""
from __future__ import annotations

import math

import torch


def _next_fast_len(n: int) -> int:
    """Smallest 2^a 3^b 5^c >= n (scipy.fftpack.next_fast_len, which the
    reference imports at diagnostics.py:18)."""
    best = None
    p5 = 1
    while p5 < 2 * n:
        p35 = p5
        while p35 < 2 * n:
            p = p35
            while p < n:
                p *= 2
            if best is None or p < best:
                best = p
            p35 *= 3
        p5 *= 5
    return best


def potential_scale_reduction(x, chain_axis=0, sample_axis=1):
    x = torch.as_tensor(x).double()
    n = x.shape[sample_axis]
    mean = x.mean(dim=sample_axis, keepdim=True)
    var = x.var(dim=sample_axis, unbiased=True, keepdim=True)
    B = n * mean.var(dim=chain_axis, unbiased=True, keepdim=True)
    W = var.mean(dim=chain_axis, keepdim=True)
    return torch.sqrt((B / W + n - 1) / n).squeeze()


def autocovariance_stats(x, chain_axis=0, sample_axis=1):
    """The sufficient statistics of the ESS over a set of chains: the sum over
    chains of each chain's centred FFT autocovariance (diagnostics.py:131-143),
    [N, ...], and the chain means, [M, ...].  Sums from disjoint sets of chains
    add, so ranks that hold different chains reduce these instead of
    gathering their traces."""
    x = torch.as_tensor(x).double()
    x = torch.movedim(x, (chain_axis, sample_axis), (0, 1))
    N = x.shape[1]
    if N < 4:
        raise ValueError("effective_sample_size needs at least four samples per chain")
    mean = x.mean(dim=1, keepdim=True)
    cen = x - mean
    m = _next_fast_len(2 * N)
    f = torch.fft.rfft(cen, n=m, dim=1)
    acov = torch.fft.irfft(f * f.conj(), n=m, dim=1)[:, :N] / N
    return acov.sum(dim=0), mean[:, 0]


def ess_from_stats(acov_sum, chain_means):
    """ESS from ``autocovariance_stats`` (diagnostics.py:144-209): mean
    autocovariance over chains, Geyer's initial positive then monotone
    sequence, τ̂ floored at 1/log10(MN), ESS = MN/τ̂."""
    M, N = chain_means.shape[0], acov_sum.shape[0]
    if M < 2:
        raise ValueError("effective_sample_size needs two or more chains")
    mean_acov = acov_sum / M
    mean_var0 = mean_acov[0] * N / (N - 1.0)
    weighted_var = mean_var0 * (N - 1.0) / N + chain_means.var(dim=0, unbiased=True)
    n_even = N - N % 2
    rho = torch.cat([torch.ones_like(mean_var0)[None],
                     1.0 - (mean_var0[None] - mean_acov[1:n_even]) / weighted_var[None]], dim=0)
    rho_even, rho_odd = rho[0::2], rho[1::2]
    T = rho_even.shape[0]
    mask0 = (rho_even + rho_odd) > 0.0
    mask = torch.cumprod(mask0.to(torch.int64), dim=0).bool()
    tt = torch.arange(T, device=acov_sum.device).view((T,) + (1,) * (mask.ndim - 1))
    max_t = torch.where(mask, tt, torch.zeros_like(tt)).max(dim=0).values
    rho_odd = torch.where(mask, rho_odd, torch.zeros_like(rho_odd))
    idx = torch.clamp(max_t + 1, max=T - 1)
    valid = (max_t + 1) < T
    sel = torch.gather(rho_even, 0, idx[None])[0] > 0
    mask_even = mask.clone()
    cur = torch.gather(mask_even, 0, idx[None])[0]
    mask_even.scatter_(0, idx[None], torch.where(valid, sel, cur)[None])
    rho_even = torch.where(mask_even, rho_even, torch.zeros_like(rho_even))
    s = rho_even + rho_odd
    # monotone sequence: running minimum
    run = torch.cummin(s, dim=0).values
    upd = s > torch.cat([s[:1], run[:-1]], dim=0)
    rho_even_f = torch.where(upd, run / 2.0, rho_even)
    rho_odd_f = torch.where(upd, run / 2.0, rho_odd)
    ess_raw = M * N
    last = torch.gather(rho_even_f, 0, idx[None])[0]
    tau = -1.0 + 2.0 * torch.sum(rho_even_f + rho_odd_f, dim=0) - last
    tau = torch.clamp(tau, min=1.0 / math.log10(ess_raw))
    return (ess_raw / tau).squeeze()


def effective_sample_size(x, chain_axis=0, sample_axis=1):
    x = torch.as_tensor(x)
    if x.shape[chain_axis] < 2:
        raise ValueError("effective_sample_size needs two or more chains")
    return ess_from_stats(*autocovariance_stats(x, chain_axis, sample_axis))


ess = effective_sample_size
rhat = potential_scale_reduction
