"""The device ESS / R-hat (torch on CUDA tensors, cuFFT) against the oracle's
NumPy restatement of diagnostics.py:25-209, including the trace shape the
min-ESS/s measurement uses ([transitions, chains, d] = [200, 4096, 25])."""
import numpy as np
import pytest
import torch

from geomjax_gb300 import diagnostics as D
from oracle import diagnostics as OD

pytestmark = pytest.mark.gpu


def _ar1(shape, sa, seed, phi=0.7):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape)
    out = np.empty_like(x)
    sl = [slice(None)] * len(shape)
    prev = None
    for k in range(shape[sa]):
        sl[sa] = k
        cur = x[tuple(sl)] if prev is None else phi * prev + x[tuple(sl)]
        out[tuple(sl)] = cur
        prev = cur
    return out


@pytest.mark.parametrize("shape,ca,sa", [((4, 500, 3), 0, 1), ((300, 8, 5), 1, 0),
                                         ((2, 101), 0, 1), ((200, 4096, 25), 1, 0),
                                         ((20, 4096, 25), 1, 0)])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_device_ess_rhat_match_oracle(shape, ca, sa, dtype):
    x = _ar1(shape, sa, seed=3)
    # the device trace is float32 in the mixed form: the oracle sees the same values
    xd = torch.tensor(x, dtype=dtype, device="cuda")
    xh = xd.double().cpu().numpy()
    e1 = D.effective_sample_size(xd, chain_axis=ca, sample_axis=sa)
    assert e1.is_cuda
    e2 = OD.effective_sample_size(xh, chain_axis=ca, sample_axis=sa)
    np.testing.assert_allclose(e1.cpu().numpy(), e2, rtol=1e-9)
    r1 = D.potential_scale_reduction(xd, chain_axis=ca, sample_axis=sa)
    r2 = OD.potential_scale_reduction(xh, chain_axis=ca, sample_axis=sa)
    np.testing.assert_allclose(r1.cpu().numpy(), r2, rtol=1e-10)


def test_device_ess_of_independent_draws_is_near_the_draw_count():
    """iid N(0,1) draws: the ESS is the number of draws up to its sampling
    error, on the device as in the oracle."""
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(500, 256, 4, device="cuda", generator=g, dtype=torch.float64)
    e = D.effective_sample_size(x, chain_axis=1, sample_axis=0).cpu().numpy()
    e2 = OD.effective_sample_size(x.cpu().numpy(), chain_axis=1, sample_axis=0)
    np.testing.assert_allclose(e, e2, rtol=1e-9)
    assert np.all(np.abs(e / (500 * 256) - 1) < 0.1)
