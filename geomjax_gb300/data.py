"""Synthetic, seeded inputs of the benchmark configurations (the reference
names no dataset for this path)."""
from __future__ import annotations

import numpy as np


def logreg_data(N: int, d: int, seed: int = 0):
    """X iid N(0, 1) rounded to float32, β* ~ N(0, I), y ~ Bernoulli(σ(Xβ*)),
    numpy PCG64(seed).  Returns float64 arrays holding the float32 values of X."""
    rng = np.random.Generator(np.random.PCG64(seed))
    X = rng.standard_normal((N, d)).astype(np.float32).astype(np.float64)
    beta = rng.standard_normal(d)
    p = 0.5 * (1.0 + np.tanh(0.5 * (X @ beta)))
    y = (rng.random(N) < p).astype(np.float64)
    return X, y


def uneven_logreg_batch(num_posteriors: int, n_range=(200, 5000), d_range=(8, 128), seed: int = 0):
    """Sizes of the uneven batch: N and d log-uniform in the given ranges."""
    rng = np.random.Generator(np.random.PCG64(seed))
    N = np.floor(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]), num_posteriors))).astype(int)
    d = np.floor(np.exp(rng.uniform(np.log(d_range[0]), np.log(d_range[1]), num_posteriors))).astype(int)
    return N, d
