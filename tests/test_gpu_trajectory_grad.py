"""Differentiated RMHMC transition (generalized leapfrog, logistic
regression), ``gj_logreg_gl_transition_jvp``.

* The primal values (p_accept, ΔH) match the float64 oracle's generalized
  leapfrog run with the same fixed number of fixed-point evaluations
  (tol = 0, max_iters = K − 1: one eager evaluation plus K − 1 more).
* The forward-mode tangents ∂/∂h and ∂/∂λ of ΔH and of p_accept match
  central finite differences (relative step 1e-4, float64) to 1e-4,
  normwise over the chains: max|J − FD| / max|FD|.
* The torch.autograd.Function wrapper returns the chain-mean Jacobian.
"""
import numpy as np
import pytest

from helpers import device_target, oracle_target, start_positions

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

N, D, C = 120, 5, 48
PRIOR_VAR = 100.0


def _inputs(C=C, seed=3):
    q0 = start_positions(D, C, seed=seed, scale=0.3)
    z = np.random.default_rng(seed + 1).standard_normal((C, D))
    return q0, z


def _normwise(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("L,K", [(1, 6), (6, 4)])
def test_primal_matches_oracle_generalized_leapfrog(L, K):
    from geomjax_gb300 import autodiff as AD
    from oracle import rmhmc as OR

    ot = oracle_target("logreg", N=N, d=D, prior_var=PRIOR_VAR)
    tg = device_target("logreg", "fp64", N=N, d=D, prior_var=PRIOR_VAR)
    q0, z = _inputs()
    h = 0.08
    pa, dH = (x.cpu().numpy() for x in AD.transition_values(tg, q0, z, h, 1.0 / PRIOR_VAR, L, K, K))
    s0 = OR.init(ot, q0)
    _, info = OR.kernel(ot, s0, z, np.full(C, -1.0), h, L, integrator="generalized_leapfrog",
                        tol=0.0, max_iters=K - 1)
    p = OR.momentum_from_normals(ot, q0, z)
    H0 = -s0.logdensity + OR.kinetic_energy(ot, q0, p)
    ref_dH = info.energy - H0
    assert np.max(np.abs(dH - ref_dH)) < 1e-9 * (1.0 + np.max(np.abs(H0)))
    np.testing.assert_allclose(pa, info.acceptance_rate, rtol=1e-8, atol=1e-12)


@pytest.mark.parametrize("L", [1, 20])
def test_tangents_match_central_differences(L):
    from geomjax_gb300 import autodiff as AD

    tg = device_target("logreg", "fp64", N=N, d=D, prior_var=PRIOR_VAR)
    q0, z = _inputs()
    h, lam, e = 0.08, 0.5, 1e-4
    J = AD.transition_jacobian(tg, q0, z, h, lam, L).cpu().numpy()

    def vals(hh, ll):
        return [x.cpu().numpy() for x in AD.transition_values(tg, q0, z, hh, ll, L)]

    ph, dh = vals(h * (1 + e), lam)
    mh, mdh = vals(h * (1 - e), lam)
    pl, dl = vals(h, lam * (1 + e))
    ml, mdl = vals(h, lam * (1 - e))
    assert _normwise(J[:, 4], (dh - mdh) / (2 * e * h)) < 1e-4
    assert _normwise(J[:, 5], (dl - mdl) / (2 * e * lam)) < 1e-4
    # p_accept = min(exp(−ΔH), 1) is smooth only where it is not clipped
    smooth = J[:, 3] > 1e-3
    if smooth.sum() >= 2:
        assert _normwise(J[smooth, 1], ((ph - mh) / (2 * e * h))[smooth]) < 1e-4
        assert _normwise(J[smooth, 2], ((pl - ml) / (2 * e * lam))[smooth]) < 1e-4
    assert np.all(J[~smooth & (J[:, 0] == 1.0), 1] == 0.0)


def test_autograd_function_returns_mean_jacobian():
    from geomjax_gb300 import autodiff as AD

    tg = device_target("logreg", "fp64", N=N, d=D, prior_var=PRIOR_VAR)
    q0, z = _inputs(C=32)
    h = torch.tensor(0.08, dtype=torch.float64, requires_grad=True)
    lam = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    pa, dH = AD.transition_stats(tg, q0, z, h, lam, 10)
    (pa + 2.0 * dH).backward()
    J = AD.transition_jacobian(tg, q0, z, 0.08, 0.5, 10).mean(dim=0).cpu()
    assert torch.allclose(h.grad.cpu(), J[1] + 2.0 * J[4], rtol=1e-12)
    assert torch.allclose(lam.grad.cpu(), J[2] + 2.0 * J[5], rtol=1e-12)


def test_rejects_unsupported():
    from geomjax_gb300 import _lib as L
    from geomjax_gb300 import autodiff as AD

    tg = device_target("logreg", "mixed", N=N, d=D)
    with pytest.raises(ValueError):
        AD.transition_stats(tg, *_inputs(C=4), 0.1, 0.5, 2)
    big = device_target("logreg", "fp64", N=40, d=70)
    with pytest.raises(L.GeomjaxError):
        AD.transition_values(big, np.zeros((2, 70)), np.zeros((2, 70)), 0.1, 0.5, 1)


def test_full_size_config_tangents_match_central_differences():
    """The config's size: N = 2000, d = 64, L = 20 generalized-leapfrog steps
    (here on 32 chains; the cost per chain does not depend on the chain
    count).  ∂ΔH/∂h at the config's λ = 1/100, and ∂ΔH/∂λ at λ = 50, against
    central differences (relative step 1e-4, float64), normwise 1e-4.  At
    λ = 1/100 the regulariser is 2e-5 of G's scale (≈ 500·I), so ∂ΔH/∂λ is
    below the float64 resolution of H ≈ 10³ and is only checked finite."""
    from geomjax_gb300 import autodiff as AD
    from geomjax_gb300.data import logreg_data

    import geomjax_gb300 as gj

    X, y = logreg_data(2000, 64, seed=0)
    tg = gj.logistic_regression(X, y, precision="fp64")
    Cc = 32
    rng = np.random.default_rng(5)
    q0 = 0.05 * rng.standard_normal((Cc, 64))
    z = rng.standard_normal((Cc, 64))
    h, e, L = 0.02, 1e-4, 20

    def dH(hh, ll):
        return AD.transition_values(tg, q0, z, hh, ll, L)[1].cpu().numpy()

    lam = 0.01
    J = AD.transition_jacobian(tg, q0, z, h, lam, L).cpu().numpy()
    assert np.all(np.isfinite(J))
    fd_h = (dH(h * (1 + e), lam) - dH(h * (1 - e), lam)) / (2 * e * h)
    assert _normwise(J[:, 4], fd_h) < 1e-4
    lam = 50.0
    J = AD.transition_jacobian(tg, q0, z, h, lam, L).cpu().numpy()
    fd_l = (dH(h, lam * (1 + e)) - dH(h, lam * (1 - e))) / (2 * e * lam)
    assert _normwise(J[:, 5], fd_l) < 1e-4


def test_gradient_step_size_adaptation_hits_target_acceptance():
    """Newton iterations on ⟨p_accept⟩(h) with the exact derivative reach the
    target acceptance on the common momentum draws."""
    from geomjax_gb300.adaptation import gradient_step_size_adaptation

    tg = device_target("logreg", "fp64", N=N, d=D, prior_var=PRIOR_VAR)
    q0, _ = _inputs(C=64)
    res = gradient_step_size_adaptation(tg, q0, 10, initial_step_size=0.05,
                                        target_acceptance_rate=0.8, num_iterations=40, tol=1e-4)
    # within tol of the target, or at a jump where one of the 64 chains starts
    # to diverge (at most 1/64 of the mean)
    assert abs(res.mean_acceptance - 0.8) < 1.0 / 64, res
    assert res.step_size > 0.05  # 0.05 accepts nearly everything here
    assert all(np.isfinite(hd) for _, _, hd in res.history)
    assert res.iterations < 40
