"""Iterative NUTS on the device (``gj_nuts_step``) with the RMHMC, dense-LMC
and LMC-Monge dynamics, against the float64 oracle's per-chain restatement
of rmhmc/nuts.py, lmcmc/nuts.py and lmcmonge/nuts.py.

FP64: positions, log densities, energies and acceptance rates to 1e-9
(e = max |gpu − oracle| / (1 + |oracle|)); the discrete outcomes (number of
expansions, of integration steps, U-turn and divergence flags) exactly; three
chained transitions of 8 chains with up to 2^6 steps each.  A stationarity
check runs 4096 chains started at the funnel's exact distribution through
20 transitions and keeps v ~ N(0, 9).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import nuts as ON  # noqa: E402
from oracle import rmhmc as O_rm  # noqa: E402
from tests.helpers import device_target, oracle_target, rel_err, start_positions  # noqa: E402

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().double().cpu().numpy()


@pytest.mark.parametrize("integrator,criterion", [("implicit_midpoint", "euc"),
                                                  ("generalized_leapfrog", "euc"),
                                                  ("implicit_midpoint", "bet"),
                                                  ("implicit_midpoint", "riem")])
@pytest.mark.parametrize("kind,kw,h", [
    ("funnel", dict(D=2, metric="diag"), 0.2),
    ("funnel", dict(D=4, metric="pullback"), 0.15),
    ("hier", dict(J=3), 0.2),
    ("logreg", dict(N=30, d=3), 0.3),
], ids=str)
def test_nuts_matches_oracle(kind, kw, h, integrator, criterion):
    import geomjax_gb300 as gj

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, "fp64", **kw)
    C, M = 8, 6
    q0 = start_positions(ot.dim, C, seed=1, scale=0.5)
    kern = gj.nutsrmhmc.build_kernel(integrator=integrator)
    st = gj.nutsrmhmc.init(q0, dt)
    so = O_rm.init(ot, q0)
    rng = np.random.Generator(np.random.PCG64(11))
    for t in range(3):
        z = rng.standard_normal((C, ot.dim))
        u = rng.random((C, ON.num_uniforms(M)))
        so, oinfo = ON.kernel(ot, so, z, u, h, M, integrator=integrator, criterion=criterion)
        st, info = kern(gj.NUTSDraws(z, u), st, dt, h, M, stopping_criterion=criterion)
        np.testing.assert_array_equal(_np(info.num_integration_steps),
                                      [i.num_integration_steps for i in oinfo])
        np.testing.assert_array_equal(_np(info.num_trajectory_expansions),
                                      [i.num_trajectory_expansions for i in oinfo])
        np.testing.assert_array_equal(_np(info.is_turning).astype(bool),
                                      [i.is_turning for i in oinfo])
        np.testing.assert_array_equal(_np(info.is_divergent).astype(bool),
                                      [i.is_divergent for i in oinfo])
        assert rel_err(_np(st.position), so.position) < 1e-9, t
        assert rel_err(_np(st.logdensity), so.logdensity) < 1e-9
        assert rel_err(_np(info.acceptance_rate), [i.acceptance_rate for i in oinfo]) < 1e-9
        assert rel_err(_np(info.energy), [i.energy for i in oinfo]) < 1e-9
        # a divergent chain's extreme is the state that diverged: compare the rest
        ok = ~np.array([i.is_divergent for i in oinfo])
        assert rel_err(_np(info.trajectory_leftmost_position)[ok],
                       np.array([i.left.q for i in oinfo])[ok]) < 1e-9
        assert rel_err(_np(info.trajectory_rightmost_position)[ok],
                       np.array([i.right.q for i in oinfo])[ok]) < 1e-9


@pytest.mark.parametrize("criterion", ["euc", "bet", "riem"])
@pytest.mark.parametrize("dynamics,kind,kw,h", [
    ("lmc", "funnel", dict(D=3, metric="pullback"), 0.1),
    ("lmc", "hier", dict(J=3), 0.1),
    ("lmcmonge", "funnel", dict(D=5, metric="diag"), 0.05),
    ("lmcmonge", "hier", dict(J=4), 0.05),
], ids=str)
def test_lmc_nuts_matches_oracle(dynamics, kind, kw, h, criterion):
    import geomjax_gb300 as gj
    from oracle import lmc as O_lmc
    from oracle import lmcmonge as O_mo

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, "fp64", **kw)
    C, M, d = 8, 6, ot.dim
    q0 = start_positions(d, C, seed=2, scale=0.5)
    im = np.linspace(0.9, 1.1, d)
    a2 = 0.5
    if dynamics == "lmc":
        kern = gj.nutslmc.build_kernel()
        st = gj.nutslmc.init(q0, dt)
        so = O_lmc.init(ot, q0)
        okw = {}
    else:
        kern0 = gj.nutslmcmonge.build_kernel(max_num_doublings=M)
        imt = torch.as_tensor(im, device="cuda")

        def kern(key, s, t, hh, MM, stopping_criterion):
            return kern0(key, s, t, hh, imt, a2, stopping_criterion)
        st = gj.nutslmcmonge.init(q0, dt)
        so = O_mo.init(ot, q0)
        okw = dict(alpha2=a2, inverse_mass_matrix=im)
    rng = np.random.Generator(np.random.PCG64(13))
    for t in range(3):
        z = rng.standard_normal((C, d))
        u = rng.random((C, ON.num_uniforms(M)))
        so, oinfo = ON.kernel(ot, so, z, u, h, M, dynamics=dynamics, criterion=criterion, **okw)
        st, info = kern(gj.NUTSDraws(z, u), st, dt, h, M, stopping_criterion=criterion)
        np.testing.assert_array_equal(_np(info.num_integration_steps),
                                      [i.num_integration_steps for i in oinfo])
        np.testing.assert_array_equal(_np(info.num_trajectory_expansions),
                                      [i.num_trajectory_expansions for i in oinfo])
        np.testing.assert_array_equal(_np(info.is_turning).astype(bool),
                                      [i.is_turning for i in oinfo])
        assert rel_err(_np(st.position), so.position) < 1e-9, t
        assert rel_err(_np(st.volume_adjustment), so.volume_adjustment) < 1e-9
        assert rel_err(_np(st.logdensity_grad), so.logdensity_grad) < 1e-9
        assert rel_err(_np(info.acceptance_rate), [i.acceptance_rate for i in oinfo]) < 1e-9
        assert rel_err(_np(info.energy), [i.energy for i in oinfo]) < 1e-9


def test_nuts_keeps_the_funnel_stationary():
    import geomjax_gb300 as gj

    dt = device_target("funnel", "fp64", D=2, metric="diag")
    C = 4096
    rng = np.random.default_rng(0)
    v = 3.0 * rng.standard_normal(C)
    x = np.exp(v / 2) * rng.standard_normal(C)
    alg = gj.nutsrmhmc(dt, 0.2, max_num_doublings=8)
    st = alg.init(np.stack([x, v], axis=1))
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    steps = []
    for _ in range(20):
        st, info = alg.step(gen, st)
        steps.append(_np(info.num_integration_steps).mean())
    vv = _np(st.position)[:, 1]
    assert abs(vv.mean()) < 0.3, vv.mean()  # SE 3/√4096 ≈ 0.05
    assert abs(vv.var() - 9.0) < 1.5, vv.var()  # SE ≈ 0.2
    assert np.mean(steps) > 2


def test_nuts_mixed_precision_runs():
    import geomjax_gb300 as gj

    dt = device_target("logreg", "mixed", N=100, d=5, seed=2)
    alg = gj.nutsrmhmc(dt, 0.3, max_num_doublings=6)
    st = alg.init(start_positions(5, 256, seed=3, scale=0.2))
    for s in range(3):
        st, info = alg.step(s, st)
    assert np.isfinite(_np(st.position)).all()
    assert (_np(info.num_integration_steps) >= 1).all()
    assert 0.0 < _np(info.acceptance_rate).mean() <= 1.0


def test_nuts_argument_checks():
    import geomjax_gb300 as gj
    from geomjax_gb300 import _lib as L

    dt = device_target("funnel", "fp64", D=2, metric="diag")
    st = gj.nutsrmhmc.init(np.ones((4, 2)), dt)
    kern = gj.nutsrmhmc.build_kernel()
    with pytest.raises(L.GeomjaxError):
        kern(0, st, dt, 0.1, 17)
    with pytest.raises(ValueError):
        kern(gj.NUTSDraws(np.zeros((4, 2)), np.zeros((4, 5))), st, dt, 0.1, 3)
    with pytest.raises(ValueError):
        kern(0, st, dt, 0.1, 3, stopping_criterion="x")


def test_nuts_lmcmonge_mixed_precision_runs():
    """The float32 Monge dynamics (D = 20 funnel, α² = 1) through NUTS."""
    import geomjax_gb300 as gj

    dt = device_target("funnel", "mixed", D=20, metric="diag")
    alg = gj.nutslmcmonge(dt, 0.05, torch.ones(20, device="cuda"), alpha2=1.0,
                          max_num_doublings=6)
    st = alg.init(np.ones((512, 20)))
    for s in range(3):
        st, info = alg.step(s, st)
    assert np.isfinite(_np(st.position)).all()
    assert np.isfinite(_np(st.volume_adjustment)).all()
    assert (_np(info.num_integration_steps) >= 1).all()
    assert 0.0 < _np(info.acceptance_rate).mean() <= 1.0
