"""MCMC diagnostics (float64 NumPy).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Restates ``diagnostics.py:25-75`` (potential_scale_reduction) and
``diagnostics.py:78-209`` (effective_sample_size: FFT autocovariance padded
to ``next_fast_len(2n)``, Geyer's initial positive sequence, then the
initial monotone sequence, τ̂ floored at 1/log10(MN), ESS = MN/τ̂).
"""
from __future__ import annotations

import numpy as np
from scipy.fftpack import next_fast_len  # the reference imports this one (diagnostics.py:18)


def potential_scale_reduction(x, chain_axis=0, sample_axis=1):
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[sample_axis]
    mean = x.mean(axis=sample_axis, keepdims=True)
    var = x.var(axis=sample_axis, ddof=1, keepdims=True)
    B = n * mean.var(axis=chain_axis, ddof=1, keepdims=True)
    W = var.mean(axis=chain_axis, keepdims=True)
    return np.sqrt((B / W + n - 1) / n).squeeze()


def effective_sample_size(x, chain_axis=0, sample_axis=1):
    x = np.asarray(x, dtype=np.float64)
    # move to [chains, samples, rest...]
    x = np.moveaxis(x, (chain_axis, sample_axis), (0, 1))
    M, N = x.shape[0], x.shape[1]
    assert M > 1, "effective_sample_size needs two or more chains"
    mean = x.mean(axis=1, keepdims=True)
    cen = x - mean
    m = next_fast_len(2 * N)
    f = np.fft.rfft(cen, n=m, axis=1)
    f = f * np.conjugate(f)
    acov = np.fft.irfft(f, n=m, axis=1)[:, :N] / N
    mean_acov = acov.mean(axis=0)  # [N, rest...]
    mean_var0 = mean_acov[0] * N / (N - 1.0)
    weighted_var = mean_var0 * (N - 1.0) / N + mean[:, 0].var(axis=0, ddof=1)
    n_even = N - N % 2
    rho = np.concatenate([np.ones_like(mean_var0)[None],
                          1.0 - (mean_var0[None] - mean_acov[1:n_even]) / weighted_var[None]], axis=0)
    rho_even = rho[0::2]
    rho_odd = rho[1::2]
    # Geyer's initial positive sequence (diagnostics.py:164-182)
    mask0 = (rho_even + rho_odd) > 0.0
    mask = np.cumprod(mask0, axis=0).astype(bool)
    T = mask0.shape[0]
    max_t = np.where(mask, np.arange(T).reshape((T,) + (1,) * (mask.ndim - 1)), 0).max(axis=0)
    max_t = np.where(mask.any(axis=0), max_t, 0)
    rho_odd = np.where(mask, rho_odd, 0.0)
    mask_even = mask.copy()
    idx = np.minimum(max_t + 1, T - 1)  # JAX clamps out-of-range scatter/gather indices
    sel = np.take_along_axis(rho_even, idx[None], axis=0)[0] > 0
    valid = (max_t + 1) < T
    np.put_along_axis(mask_even, idx[None], np.where(valid, sel, np.take_along_axis(mask_even, idx[None], 0)[0])[None], axis=0)
    rho_even = np.where(mask_even, rho_even, 0.0)
    # Geyer's initial monotone sequence (diagnostics.py:185-196)
    s = rho_even + rho_odd
    prev = s[0].copy()
    upd = np.zeros_like(mask)
    val = np.zeros_like(s)
    for t in range(T):
        u = s[t] > prev
        nv = np.where(u, prev, s[t])
        upd[t] = u
        val[t] = nv
        prev = nv
    rho_even_f = np.where(upd, val / 2.0, rho_even)
    rho_odd_f = np.where(upd, val / 2.0, rho_odd)
    ess_raw = M * N
    last = np.take_along_axis(rho_even_f, idx[None], axis=0)[0]
    tau = -1.0 + 2.0 * np.sum(rho_even_f + rho_odd_f, axis=0) - last
    tau = np.maximum(tau, 1.0 / np.log10(ess_raw))
    return (ess_raw / tau).squeeze()
