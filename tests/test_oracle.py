"""Checks of the float64 oracle itself (CPU only).

* analytic ∇ℓ, HVP, ∂G against central finite differences;
* the reference's structural pins (``tests/test_samplers.py:21-57``):
  RMHMC with G = I ≡ HMC velocity Verlet ≡ dense LMC with G = I (rtol 1e-4);
* the closed-form Monge velocity factor against the reference's dense
  Cholesky (``lmcmonge/metrics.py:155-166``);
* reversibility under momentum flip and the O(h²) energy error.
"""
import numpy as np
import pytest

from oracle import targets as T
from oracle import rmhmc, lmcmonge, lmc, hmc, diagnostics


def _targets():
    X, y = T.make_logreg_data(40, 5, seed=1)
    yh, sh = T.make_hier_data(6, seed=2)
    return [
        T.Funnel(D=2, metric="diag"),
        T.Funnel(D=5, metric="diag"),
        T.Funnel(D=4, metric="pullback"),
        T.LogisticRegression(X, y),
        T.HierarchicalGaussian(yh, sh),
    ]


def _q(tg, C=3, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((C, tg.dim)) * 0.5


@pytest.mark.parametrize("tg", _targets(), ids=lambda t: f"{t.family}-{t.dim}")
def test_grad_hvp_metric_fd(tg):
    q = _q(tg)
    eps = 1e-6
    g = tg.grad(q)
    rng = np.random.default_rng(5)
    u = rng.standard_normal(q.shape)
    Hu = tg.hvp(q, u)
    G = tg.metric(q)
    dG = tg.dmetric(q)
    for k in range(tg.dim):
        e = np.zeros(tg.dim)
        e[k] = eps
        fd = (tg.logdensity(q + e) - tg.logdensity(q - e)) / (2 * eps)
        np.testing.assert_allclose(g[:, k], fd, rtol=1e-6, atol=1e-6)
        fdG = (tg.metric(q + e) - tg.metric(q - e)) / (2 * eps)
        np.testing.assert_allclose(dG[..., k], fdG, rtol=1e-6, atol=1e-6)
    fdH = (tg.grad(q + eps * u) - tg.grad(q - eps * u)) / (2 * eps)
    np.testing.assert_allclose(Hu, fdH, rtol=1e-5, atol=1e-5)
    if not tg.is_diagonal:
        np.testing.assert_allclose(G, np.swapaxes(G, 1, 2))
        assert np.all(np.linalg.eigvalsh(G) > 0)


def test_logreg_structured_contractions():
    X, y = T.make_logreg_data(30, 4, seed=3)
    tg = T.LogisticRegression(X, y)
    q = _q(tg)
    G = tg.metric(q)
    Ginv = np.linalg.inv(G)
    u = np.random.default_rng(0).standard_normal(q.shape)
    tr, quad = tg.metric_trace_quad(q, Ginv, u)
    dG = tg.dmetric(q)
    np.testing.assert_allclose(tr, np.einsum("cab,cbak->ck", Ginv, dG), rtol=1e-10)
    np.testing.assert_allclose(quad, np.einsum("ca,cabk,cb->ck", u, dG, u), rtol=1e-10)
    np.testing.assert_allclose(tg.dmetric_vec(q, u), np.einsum("cabk,ck->cab", dG, u), rtol=1e-10)


def test_lmc_logreg_structured_omega_matches_einsums():
    """The dense-LMC oracle's logistic-regression shortcut (Ω̃ = G + h/4·Σ_i
    v_i ∂_iG, tr(G⁻¹∂_kG) from the per-datum form) equals the three einsums of
    lmcmc/metrics.py:174-176 and the trace of :181-189 over the full ∂G."""
    X, y = T.make_logreg_data(40, 5, seed=4)
    tg = T.LogisticRegression(X, y)
    q = _q(tg)
    v = np.random.default_rng(1).standard_normal(q.shape)
    dG = tg.dmetric(q)
    G = tg.metric(q)
    for h in (0.1, -0.1):
        p1 = np.einsum("ci,cjli->clj", v, dG)
        p2 = np.einsum("ci,cilj->clj", v, dG)
        p3 = np.einsum("ci,cijl->clj", v, dG)
        full = G + 0.5 * h * 0.5 * (p1 + p2 - p3)
        np.testing.assert_allclose(lmc.omega_tilde(tg, q, v, h), full, rtol=1e-12, atol=1e-12)
    tr_full = np.einsum("cab,cbak->ck", np.linalg.inv(G), dG)
    np.testing.assert_allclose(lmc.grad_logdetmetric(tg, q), tr_full, rtol=1e-10)


def test_kinetic_grad_fd():
    for tg in _targets():
        q = _q(tg)
        p = np.random.default_rng(1).standard_normal(q.shape)
        dq, dp = rmhmc.kinetic_grad(tg, q, p)
        eps = 1e-6
        for k in range(tg.dim):
            e = np.zeros(tg.dim)
            e[k] = eps
            fd = (rmhmc.kinetic_energy(tg, q + e, p) - rmhmc.kinetic_energy(tg, q - e, p)) / (2 * eps)
            np.testing.assert_allclose(dq[:, k], fd, rtol=1e-5, atol=1e-6)
            fdp = (rmhmc.kinetic_energy(tg, q, p + e) - rmhmc.kinetic_energy(tg, q, p - e)) / (2 * eps)
            np.testing.assert_allclose(dp[:, k], fdp, rtol=1e-5, atol=1e-6)


def test_reference_structural_pin_identity_metric():
    """tests/test_samplers.py:21-57: rmhmc(G=I) ≈ hmc(ones) ≈ lmc(G=I), rtol 1e-4,
    step 1e-2, 10 steps, same momenta, from zeros(2) on the funnel."""
    base = T.Funnel(D=2)
    tg = T.IdentityMetric(base)
    C = 16
    rng = np.random.default_rng(42)
    z = rng.standard_normal((C, 2))
    u = rng.random(C)
    q0 = np.zeros((C, 2))
    s = rmhmc.init(tg, q0)
    s1, _ = rmhmc.kernel(tg, s, z, u, 1e-2, 10)
    q2, _ = hmc.kernel(base, q0, z, u, 1e-2, 10)
    s3, _ = lmc.kernel(tg, lmc.init(tg, q0), z, u, 1e-2, 10)
    np.testing.assert_allclose(s1.position, q2, rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(q2, s3.position, rtol=1e-4, atol=1e-7)
    # generalized leapfrog at G = I is leapfrog too
    s4, _ = rmhmc.kernel(tg, s, z, u, 1e-2, 10, integrator="generalized_leapfrog")
    np.testing.assert_allclose(s4.position, q2, rtol=1e-4, atol=1e-7)


def test_monge_alpha0_quirk():
    """At α² = 0 the Monge metric is M and the Lan integrator should be
    leapfrog.  The reference's half_step_omega omits α² in its
    Sherman-Morrison correction (lmcmonge/integrators.py:186-189), so with
    the reference form it does NOT match HMC — exactly the commented-out
    assertion "Monge does not match" (tests/test_samplers.py:58-59).  With
    the α²-consistent form it matches."""
    base = T.Funnel(D=2)
    C = 8
    rng = np.random.default_rng(3)
    z = rng.standard_normal((C, 2))
    u = np.zeros(C)
    q0 = rng.standard_normal((C, 2)) * 0.3
    q2, _ = hmc.kernel(base, q0, z, u, 1e-2, 10)
    s1, _ = lmcmonge.kernel(base, lmcmonge.init(base, q0), z, u, 1e-2, np.ones(2), 10, alpha2=0.0)
    assert not np.allclose(s1.position, q2, rtol=1e-4)
    s2, _ = lmcmonge.kernel(base, lmcmonge.init(base, q0), z, u, 1e-2, np.ones(2), 10, alpha2=0.0,
                            alpha2_fix=True)
    np.testing.assert_allclose(s2.position, q2, rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("alpha2", [1.0, 0.3, 1e-3])
def test_monge_closed_form_velocity(alpha2):
    rng = np.random.default_rng(7)
    C, d = 5, 17
    g = rng.standard_normal((C, d)) * 3
    inv_mass = rng.uniform(0.5, 2.0, d)
    L = lmcmonge.normalizing_constant(alpha2, inv_mass, g)
    dl_ig = inv_mass * g / np.sqrt(L)[:, None]
    z = rng.standard_normal((C, d))
    a = lmcmonge.velocity_dense(alpha2, inv_mass, dl_ig, z)
    b = lmcmonge.velocity_closed_form(alpha2, inv_mass, dl_ig, z, L)
    np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12)


def _energy_err(kind, tg, h, L=None):
    rng = np.random.default_rng(11)
    C = 6
    q0 = _q(tg, C, seed=4) * 0.5
    z = rng.standard_normal((C, tg.dim))
    u = np.zeros(C)
    if L is None:
        L = max(1, int(round(0.4 / h)))
    if kind == "rmhmc":
        _, info = rmhmc.kernel(tg, rmhmc.init(tg, q0), z, u, h, L, tol=1e-12)
    elif kind == "rmhmc_gl":
        _, info = rmhmc.kernel(tg, rmhmc.init(tg, q0), z, u, h, L, tol=1e-12, integrator="generalized_leapfrog")
    elif kind == "lmc":
        _, info = lmc.kernel(tg, lmc.init(tg, q0), z, u, h, L)
    else:
        _, info = lmcmonge.kernel(tg, lmcmonge.init(tg, q0), z, u, h, np.ones(tg.dim), L, alpha2=1.0)
    return np.max(np.abs(np.log(np.maximum(info.acceptance_rate, 1e-300))))


@pytest.mark.parametrize("kind", ["rmhmc", "rmhmc_gl", "lmc", "monge"])
def test_energy_error_shrinks_quadratically(kind):
    """Over a fixed time 0.4 the energy error of a 2nd-order integrator drops
    ~4× when h halves (only the acceptance-side error |min(w,0)| is visible,
    so chains are checked in aggregate)."""
    yh, sh = T.make_hier_data(3, seed=2)
    tg = T.HierarchicalGaussian(yh, sh) if kind != "monge" else T.Funnel(D=4)
    e1 = _energy_err(kind, tg, 0.04)
    e2 = _energy_err(kind, tg, 0.02)
    assert e2 < e1 / 2.5 or e1 < 1e-9


def test_rmhmc_reversible():
    tg = T.Funnel(D=3, metric="pullback")
    q0 = _q(tg, 4)
    z = np.random.default_rng(9).standard_normal(q0.shape)
    s = rmhmc.init(tg, q0)
    p = rmhmc.momentum_from_normals(tg, q0, z)
    st = rmhmc.IntegratorState(q0, p, rmhmc.inverse_metric_vector_product(tg, q0, p), s.logdensity, s.logdensity_grad)
    for _ in range(5):
        st, _ = rmhmc.implicit_midpoint_step(tg, st, 0.05, tol=1e-13)
    st = rmhmc.IntegratorState(st.position, -st.momentum, -st.velocity, st.logdensity, st.logdensity_grad)
    for _ in range(5):
        st, _ = rmhmc.implicit_midpoint_step(tg, st, 0.05, tol=1e-13)
    np.testing.assert_allclose(st.position, q0, atol=1e-9)
    np.testing.assert_allclose(-st.momentum, p, atol=1e-9)


def test_ess_rhat_shapes_and_iid():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((4, 2000, 3))  # chains, samples, dims
    ess = diagnostics.effective_sample_size(x, chain_axis=0, sample_axis=1)
    assert ess.shape == (3,)
    assert np.all(ess > 4000) and np.all(ess < 12000)
    rh = diagnostics.potential_scale_reduction(x)
    assert np.all(np.abs(rh - 1) < 0.01)
    # AR(1) chain with known integrated autocorrelation time (1+φ)/(1-φ)
    phi = 0.8
    y = np.zeros((8, 4000))
    e = rng.standard_normal((8, 4000))
    for t in range(1, 4000):
        y[:, t] = phi * y[:, t - 1] + e[:, t]
    ess = diagnostics.effective_sample_size(y)
    assert abs(ess - 32000 / 9.0) / (32000 / 9.0) < 0.2
