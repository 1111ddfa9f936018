"""Time reversibility of the device integrators (the oracle's own is
tests/test_oracle.py::test_rmhmc_reversible): integrate L steps, flip the
proposal's momentum (velocity), integrate L steps again from there, and the
chain is back at its start with its initial velocity (and, for LMC-Monge,
with the volume term J of the second run the negative of the first's).

* RMHMC, generalized leapfrog, on the batched mixed path: logistic
  regression N = 1000, d = 25 (the benchmark's data), 256 chains, L = 8,
  h = 0.05 (rmhmc/rmhmc.py:425-437 for the flip);
* LMC-Monge, funnel D = 100, α² = 1, 256 chains, L = 16, h = 0.02
  (lmcmonge/lmc.py:472-565 for the flip).

The flipped momentum enters the second run through its draw:
z = chol(G(q_L))⁻¹·(−p_L) for RMHMC, z = F(q_L)⁻¹·(−v_L) for LMC-Monge with
F = chol(M⁻¹ − α²·w wᵀ) the velocity factor of lmcmonge/metrics.py:155-166,
both formed in float64 from the oracle's target at q_L.  The fixed-point
solves stop at the default tolerance 1e-6 and the mixed path evaluates in
float32, so the return is checked to 5e-5 (relative, with 1 added to the
denominator); an integrator that is not reversible misses by O(h).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import targets as OT  # noqa: E402
from tests.helpers import laplace_draws, rel_err  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = 5e-5


def _np(t):
    return t.detach().double().cpu().numpy()


def _f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


def _lower_solve(Lc, b):
    return np.linalg.solve(Lc, b[..., None])[..., 0]


def test_rmhmc_generalized_leapfrog_reversible():
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws
    from geomjax_gb300.data import logreg_data

    X, y = logreg_data(1000, 25, seed=0)
    ot = OT.LogisticRegression(X, y)
    dt = gj.logistic_regression(X, y, precision="mixed")
    C, h, L = 256, 0.05, 8
    q0 = _f32(laplace_draws(ot, C, seed=21))
    z = _f32(np.random.default_rng(22).standard_normal((C, 25)))
    keep = -np.ones(C)
    kern = gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator="generalized_leapfrog")
    _, fwd = kern(Draws(z, keep), gj.rmhmc.init(q0, dt), dt, h, L)
    p0 = _np(fwd.momentum)
    qL = _np(fwd.proposal.position)
    GL = ot.metric(qL)
    p_flip = np.einsum("cij,cj->ci", GL, _np(fwd.proposal.velocity))  # −p_L = G(q_L)·(−G⁻¹p_L)
    z2 = _lower_solve(np.linalg.cholesky(GL), p_flip)
    _, bwd = kern(Draws(z2, keep), gj.rmhmc.init(qL, dt), dt, h, L)
    e_q = rel_err(_np(bwd.proposal.position), q0)
    assert e_q < TOL, e_q
    # the reversed run ends at −p0, so its flipped velocity is G(q0)⁻¹p0
    v0 = np.linalg.solve(ot.metric(q0), p0[..., None])[..., 0]
    e_v = rel_err(_np(bwd.proposal.velocity), v0)
    assert e_v < 10 * TOL, e_v


def test_lmcmonge_reversible_funnel100():
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    D, C, h, L = 100, 256, 0.02, 16
    rng = np.random.default_rng(23)
    v = 1.5 * rng.standard_normal((C, 1))
    x = rng.standard_normal((C, D - 1)) * np.exp(0.5 * v)
    q0 = _f32(np.concatenate([x, v], axis=1))
    z = _f32(rng.standard_normal((C, D)))
    keep = -np.ones(C)
    ot = OT.Funnel(D=D)
    tg = gj.funnel(D=D, precision="mixed")
    im = torch.ones(D, dtype=torch.float32, device="cuda")
    kern = gj.lmcmonge.build_kernel()
    sf, fwd = kern(Draws(z, keep), gj.lmcmonge.init(q0, tg), tg, h, L, alpha2=1.0,
                   inverse_mass_matrix=im)
    qL = _np(fwd.proposal.position)
    g = ot.grad(qL)
    w = g / np.sqrt(1.0 + np.sum(g * g, axis=1))[:, None]  # M⁻¹∇ℓ/√L with M = I
    F = np.linalg.cholesky(np.eye(D)[None] - w[:, :, None] * w[:, None, :])
    z2 = _lower_solve(F, _np(fwd.proposal.velocity))  # the flipped velocity −v_L
    sb, bwd = kern(Draws(z2, keep), gj.lmcmonge.init(qL, tg), tg, h, L, alpha2=1.0,
                   inverse_mass_matrix=im)
    e_q = rel_err(_np(bwd.proposal.position), q0)
    assert e_q < TOL, e_q
    e_v = rel_err(_np(bwd.proposal.velocity), _np(fwd.velocity))
    assert e_v < 10 * TOL, e_v
    # the volume term J (log|det| of the map) changes sign under reversal
    jf, jb = _np(sf.volume_adjustment), _np(sb.volume_adjustment)
    assert np.max(np.abs(jf + jb) / (np.abs(jf) + 1.0)) < 1e-4, np.max(np.abs(jf + jb))
