"""Failure semantics on the device, with the failures made on the host (no
GPU fault is provoked): a NaN energy is a rejection (mcmc/proposal.py:107-108),
−(H0 − H1) > 1000 flags a divergence, a fixed point that stops short or a
non-finite proposal sets the chain's status bits, and a failing chain never
changes any other chain's result."""
import numpy as np
import pytest

from tests.helpers import device_target, normals, start_positions

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _lib():
    from geomjax_gb300 import _lib as L

    return L


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rmhmc_huge_step_rejects_and_keeps_state(precision):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    dt = device_target("funnel", precision, D=5)
    C = 64
    q0 = start_positions(5, C, seed=3, scale=0.5)
    z, u = normals(C, 5, 4, np.float32 if precision == "mixed" else np.float64)
    kern = gj.rmhmc.build_kernel(max_iters=10)
    st0 = gj.rmhmc.init(q0, dt)
    st, info = kern(Draws(z, u), st0, dt, 50.0, 10)
    acc = _np(info.is_accepted)
    assert not acc.any()
    # rejected chains keep position, log density and gradient bit for bit
    np.testing.assert_array_equal(_np(st.position), _np(st0.position))
    np.testing.assert_array_equal(_np(st.logdensity), _np(st0.logdensity))
    np.testing.assert_array_equal(_np(st.logdensity_grad), _np(st0.logdensity_grad))
    # every chain is flagged: divergent, or a fixed point / energy failure
    L = _lib()
    status = _np(info.status)
    flagged = _np(info.is_divergent) | ((status & (L.GJ_CHAIN_FP_NOT_CONVERGED | L.GJ_CHAIN_NONFINITE)) != 0)
    assert flagged.all()


def test_logreg_batched_nan_chain_is_rejected_and_isolated():
    """One chain starts at NaN: it is rejected and flagged non-finite; every
    other chain is bit-identical to a run in which that chain started at a
    finite position."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    L = _lib()
    dt = device_target("logreg", "mixed", N=300, d=9, seed=3)
    C = 160
    q0 = start_positions(9, C, seed=1, scale=0.2).astype(np.float32).astype(np.float64)
    z, u = normals(C, 9, 2, np.float32)
    kern = gj.rmhmc.build_kernel(loop="graph")
    st_ok, info_ok = kern(Draws(z, u), gj.rmhmc.init(q0, dt), dt, 0.05, 6)
    bad = 37
    q1 = q0.copy()
    q1[bad, :] = np.nan
    st_nan, info_nan = kern(Draws(z, u), gj.rmhmc.init(q1, dt), dt, 0.05, 6)
    others = np.arange(C) != bad
    np.testing.assert_array_equal(_np(st_nan.position)[others], _np(st_ok.position)[others])
    np.testing.assert_array_equal(_np(st_nan.logdensity)[others], _np(st_ok.logdensity)[others])
    np.testing.assert_array_equal(_np(info_nan.is_accepted)[others], _np(info_ok.is_accepted)[others])
    assert not bool(_np(info_nan.is_accepted)[bad])
    assert _np(info_nan.status)[bad] & (L.GJ_CHAIN_NONFINITE | L.GJ_CHAIN_FP_NOT_CONVERGED)


def test_logreg_batched_huge_step_is_divergent_and_rejected():
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    dt = device_target("logreg", "mixed", N=300, d=9, seed=3)
    C = 128
    q0 = start_positions(9, C, seed=1, scale=0.2).astype(np.float32).astype(np.float64)
    z, u = normals(C, 9, 2, np.float32)
    kern = gj.rmhmc.build_kernel(loop="graph", max_iters=20)
    st0 = gj.rmhmc.init(q0, dt)
    st, info = kern(Draws(z, u), st0, dt, 5.0, 6)
    acc = _np(info.is_accepted).astype(bool)
    assert acc.mean() < 0.05
    rej = ~acc
    np.testing.assert_array_equal(_np(st.position)[rej], _np(st0.position)[rej])
    L = _lib()
    status = _np(info.status)
    flagged = _np(info.is_divergent).astype(bool) | ((status & (L.GJ_CHAIN_FP_NOT_CONVERGED | L.GJ_CHAIN_NONFINITE)) != 0)
    assert flagged[rej].mean() > 0.9


def test_lmcmonge_huge_step_rejects():
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    dt = device_target("funnel", "mixed", D=100)
    C = 256
    q0 = np.ones((C, 100))
    z, u = normals(C, 100, 6, np.float32)
    kern = gj.lmcmonge.build_kernel()
    st0 = gj.lmcmonge.init(q0, dt)
    st, info = kern(Draws(z, u), st0, dt, 10.0, 16, alpha2=1.0,
                    inverse_mass_matrix=np.ones(100))
    acc = _np(info.is_accepted).astype(bool)
    assert acc.mean() < 0.05
    rej = ~acc
    np.testing.assert_array_equal(_np(st.position)[rej], _np(st0.position)[rej])
    np.testing.assert_array_equal(_np(st.volume_adjustment)[rej], _np(st0.volume_adjustment)[rej])
