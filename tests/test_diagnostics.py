"""The package's ESS / R-hat (torch, used on device traces) against the
oracle's NumPy restatement of diagnostics.py:25-209 (CPU)."""
import numpy as np
import pytest
import torch

from geomjax_gb300 import diagnostics as D
from oracle import diagnostics as OD


@pytest.mark.parametrize("shape,ca,sa", [((4, 500, 3), 0, 1), ((300, 8, 5), 1, 0), ((2, 101), 0, 1)])
def test_ess_matches_oracle(shape, ca, sa):
    rng = np.random.default_rng(1)
    x = rng.standard_normal(shape)
    # add autocorrelation along the sample axis
    x = np.cumsum(x, axis=sa) * 0.1 + x
    e1 = D.effective_sample_size(torch.tensor(x), chain_axis=ca, sample_axis=sa).numpy()
    e2 = OD.effective_sample_size(x, chain_axis=ca, sample_axis=sa)
    np.testing.assert_allclose(e1, e2, rtol=1e-9)
    r1 = D.potential_scale_reduction(torch.tensor(x), chain_axis=ca, sample_axis=sa).numpy()
    r2 = OD.potential_scale_reduction(x, chain_axis=ca, sample_axis=sa)
    np.testing.assert_allclose(r1, r2, rtol=1e-10)


def test_next_fast_len():
    from scipy.fftpack import next_fast_len

    for n in [1, 7, 64, 97, 1000, 2001, 4099]:
        assert D._next_fast_len(n) == next_fast_len(n)
