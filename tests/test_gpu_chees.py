"""ChEES on the device: the flipped proposal every kernel writes into its
info (RMHMCInfo.proposal.state / LMCInfo.proposal.state), the cross-chain
statistics kernel, and whole warm-up runs against the oracle's.

Tolerances: statistics 1e-10 relative (float64 sums of the same inputs in
another order); proposals as the per-step parity (FP64 1e-10, mixed 1e-5);
the FP64 warm-up run's step size and trajectory length 1e-6 relative over
30 adaptation steps (dual averaging multiplies an error in the harmonic
mean by √t / γ = 20√t in log h, and the per-transition parity is 1e-10).
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import chees as OC  # noqa: E402
from oracle import lmc as O_lmc  # noqa: E402
from oracle import lmcmonge as O_monge  # noqa: E402
from oracle import rmhmc as O_rm  # noqa: E402
from tests.helpers import device_target, normals, oracle_target, rel_err, start_positions  # noqa: E402

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().double().cpu().numpy()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("C,d", [(1, 1), (37, 5), (4096, 25), (8192, 100), (300, 129)])
def test_statistics_match_oracle(C, d, dtype):
    from geomjax_gb300.chees import chees_statistics

    rng = np.random.default_rng(C + d)
    P = rng.standard_normal((C, d))
    V = rng.standard_normal((C, d))
    I = rng.standard_normal((C, d))
    D = rng.standard_normal((C, d))
    acc = rng.uniform(0.05, 1.0, C)
    div = rng.random(C) < 0.1
    if C > 1:
        div[0] = True
        P[0, :] = np.nan  # a divergent chain with a NaN proposal
        acc[0] = 0.0
    if dtype == torch.float32:
        P, V, I, D = (x.astype(np.float32).astype(np.float64) for x in (P, V, I, D))
    t = lambda x: torch.as_tensor(x, dtype=dtype, device="cuda")  # noqa: E731
    got = chees_statistics(t(P), t(V), t(I), torch.as_tensor(acc, device="cuda"),
                           torch.as_tensor(div, device="cuda"), alpha2_tangent=t(D))
    want = OC.statistics(P, V, I, acc, div, D=D)
    if div.all():
        assert all(math.isnan(x) for x in got[:2])
        return
    for a, b in zip(got, want):
        assert a == pytest.approx(b, rel=1e-10, abs=1e-12)


def test_statistics_all_divergent_and_no_flags():
    from geomjax_gb300.chees import chees_statistics

    C, d = 64, 3
    x = torch.randn(C, d, dtype=torch.float64, device="cuda")
    acc = torch.rand(C, dtype=torch.float64, device="cuda") + 0.1
    h, g, ga = chees_statistics(x, x, x * 0.5, acc, torch.ones(C, dtype=torch.bool, device="cuda"))
    assert math.isnan(h) and math.isnan(g)
    h, g, ga = chees_statistics(x, x, x * 0.5, acc, None)
    want = OC.statistics(_np(x), _np(x), _np(x) * 0.5, _np(acc), np.zeros(C, dtype=bool))
    assert h == pytest.approx(want[0], rel=1e-12) and g == pytest.approx(want[1], rel=1e-10)
    assert ga == 0.0


def _check_proposal(info, oinfo, precision, accepted_pos=None):
    tol = 1e-10 if precision == "fp64" else 1e-5
    assert rel_err(_np(info.proposal.position), oinfo.proposal.position) < tol
    assert rel_err(_np(info.proposal.velocity), oinfo.proposal.velocity) < tol * 10


@pytest.mark.parametrize("integrator", ["implicit_midpoint", "generalized_leapfrog"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind,kw", [
    ("funnel", dict(D=2, metric="diag")),
    ("funnel", dict(D=4, metric="pullback")),
    ("logreg", dict(N=40, d=4)),
], ids=lambda x: str(x))
def test_rmhmc_proposal_matches_oracle(kind, kw, precision, integrator):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, precision, **kw)
    C, h, L = 6, 0.05, 7
    q0 = start_positions(ot.dim, C, seed=4, scale=0.3)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
    z, u = normals(C, ot.dim, 5, np.float32 if precision == "mixed" else np.float64)
    _, oinfo = O_rm.kernel(ot, O_rm.init(ot, q0), z, u, h, L, integrator=integrator)
    opts = dict(logreg_path="per_chain") if kind == "logreg" else {}
    kern = gj.rmhmc.build_kernel(integrator=integrator, **opts)
    st, info = kern(Draws(z, u), gj.rmhmc.init(q0, dt), dt, h, L)
    _check_proposal(info, oinfo, precision)
    acc = _np(info.is_accepted).astype(bool)
    np.testing.assert_array_equal(_np(st.position)[acc], _np(info.proposal.position)[acc])


@pytest.mark.parametrize("loop", ["graph", "host"])
def test_batched_logreg_proposal_matches_oracle(loop):
    """The batched mixed-precision path (tcgen05 GEMMs): proposal position
    and −G⁻¹p at the proposal, within the mixed tolerance."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=200, d=8, seed=2)
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", "mixed", **kw)
    C, h, L = 160, 0.05, 4
    q0 = start_positions(8, C, seed=1, scale=0.2).astype(np.float32).astype(np.float64)
    z, u = normals(C, 8, 3, np.float32)
    _, oinfo = O_rm.kernel(ot, O_rm.init(ot, q0), z, u, h, L)
    kern = gj.rmhmc.build_kernel(loop=loop)
    st, info = kern(Draws(z, u), gj.rmhmc.init(q0, dt), dt, h, L)
    assert rel_err(_np(info.proposal.position), oinfo.proposal.position) < 1e-5
    assert rel_err(_np(info.proposal.velocity), oinfo.proposal.velocity) < 1e-4
    acc = _np(info.is_accepted).astype(bool)
    np.testing.assert_array_equal(_np(st.position)[acc], _np(info.proposal.position)[acc])


def test_batched_graph_cache_over_jittered_lengths():
    """A jittered number of steps reuses one captured graph per length: the
    graph path equals the host-driven loop bit for bit over a sequence of
    lengths that revisits earlier ones."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    dt = device_target("logreg", "mixed", N=150, d=6, seed=4)
    C = 128
    q0 = start_positions(6, C, seed=2, scale=0.2).astype(np.float32).astype(np.float64)
    kg = gj.rmhmc.build_kernel(loop="graph")
    kh = gj.rmhmc.build_kernel(loop="host")
    sg = gj.rmhmc.init(q0, dt)
    sh = gj.rmhmc.init(q0, dt)
    for i, L in enumerate([3, 1, 3, 2, 1, 3]):
        z, u = normals(C, 6, 10 + i, np.float32)
        sg, ig = kg(Draws(z, u), sg, dt, 0.05, L)
        sh, ih = kh(Draws(z, u), sh, dt, 0.05, L)
        np.testing.assert_array_equal(_np(sg.position), _np(sh.position))
        np.testing.assert_array_equal(_np(ig.proposal.velocity), _np(ih.proposal.velocity))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lmc_proposal_matches_oracle(precision):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target("funnel", D=4, metric="pullback")
    dt = device_target("funnel", precision, D=4, metric="pullback")
    C, h, L = 5, 0.05, 6
    q0 = start_positions(4, C, seed=2, scale=0.3)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
    z, u = normals(C, 4, 9, np.float32 if precision == "mixed" else np.float64)
    _, oinfo = O_lmc.kernel(ot, O_lmc.init(ot, q0), z, u, h, L)
    st, info = gj.lmc.build_kernel()(Draws(z, u), gj.lmc.init(q0, dt), dt, h, L)
    _check_proposal(info, oinfo, precision)


@pytest.mark.parametrize("precision,D", [("fp64", 7), ("mixed", 100)])
def test_lmcmonge_proposal_matches_oracle(precision, D):
    """FP64 at D = 7 and mixed at D = 100, both on the warp-per-chain kernel."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target("funnel", D=D, metric="diag")
    dt = device_target("funnel", precision, D=D, metric="diag")
    C, h, L, a2 = 9, 0.02, 8, 1.0
    q0 = start_positions(D, C, seed=5, scale=0.5)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
    z, u = normals(C, D, 11, np.float32 if precision == "mixed" else np.float64)
    im = np.ones(D)
    _, oinfo = O_monge.kernel(ot, O_monge.init(ot, q0), z, u, h, im, L, alpha2=a2)
    kern = gj.lmcmonge.build_kernel()
    st, info = kern(Draws(z, u), gj.lmcmonge.init(q0, dt), dt, h, L, alpha2=a2,
                    inverse_mass_matrix=torch.ones(D, dtype=dt.dtype, device="cuda"))
    _check_proposal(info, oinfo, precision)


def _oracle_transition(ot, draws, kernel_fn):
    def transition(i, state, h, L):
        z, u = draws[i]
        return kernel_fn(ot, state, z, u, h, L)
    return transition


def test_rmhmc_chees_run_matches_oracle():
    """30 ChEES warm-up steps of FP64 RMHMC on a logistic-regression
    posterior (N = 300, d = 9, dense Fisher metric, 64 chains), the device
    kernels and statistics against the oracle driving its own kernel with
    the same draws: every step's number of integration steps, step size and
    trajectory length agree.  (On the funnel the early dual-averaging
    steps reach h ≈ 2, where the trajectories are chaotic and no two
    implementations stay within a tolerance.)"""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    C, D, n = 64, 9, 30
    kw = dict(N=300, d=D, seed=3)
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", "fp64", **kw)
    q0 = start_positions(D, C, seed=1, scale=0.2)
    rng = np.random.Generator(np.random.PCG64(3))
    draws = [(rng.standard_normal((C, D)), rng.random(C)) for _ in range(n)]
    warm = gj.chees_adaptation(dt, C, dynamics="rmhmc", logreg_path="per_chain")
    (last, params), hist = warm.run(0, q0, 0.1, gj.adam(0.05), n,
                                    draws=[Draws(z, u) for z, u in draws])

    def okern(t, s, z, u, h, L):
        return O_rm.kernel(t, s, z, u, h, L)

    ostate, os_, ohist, olen = OC.run(_oracle_transition(ot, draws, okern), O_rm.init(ot, q0),
                                      0.1, 0.05, n)
    assert len(hist) == len(ohist) == n
    for i, (a, b) in enumerate(zip(hist, ohist)):
        assert a.num_integration_steps == olen[i], i
        assert a.adaptation_state.step_size == pytest.approx(b.step_size, rel=1e-6), i
        assert a.adaptation_state.trajectory_length == pytest.approx(b.trajectory_length,
                                                                      rel=1e-6), i
    assert rel_err(_np(last.position), ostate.position) < 1e-6
    h, T_adj = OC.final_parameters(os_)
    assert params["step_size"] == pytest.approx(h, rel=1e-6)
    bits = math.ceil(math.log2(n + 1000))  # max_sampling_steps = 1000
    assert params["integration_steps_fn"](5) == math.ceil(
        gj.chees.halton_sequence(5, bits) * T_adj)


@pytest.mark.parametrize("dynamics,kind,kw,precision", [
    ("lmc", "funnel", dict(D=4, metric="pullback"), "fp64"),
    ("rmhmc", "logreg", dict(N=300, d=9, seed=3), "mixed"),
], ids=str)
def test_chees_run_adapts(dynamics, kind, kw, precision):
    """40 warm-up steps: the moving-average step size is finite, ChEES
    lengthens the trajectory it starts with (T₀ = h₀, one integration
    step), and the adapted dynamic kernel samples.

    The reference's statistic is fragile by construction: one chain with a
    tiny acceptance probability drags the harmonic mean down, the
    un-averaged dual-averaging iterate swings between small and large steps,
    and a step at which every chain diverges gives a NaN harmonic mean after
    which the state (and so the step size) is kept, for good
    (chees_adaptation_riemanian.py:145-154).  On this logistic regression
    with 256 chains that happens after ~55 steps, in the oracle too; the
    run here stops before it."""
    import geomjax_gb300 as gj

    dt = device_target(kind, precision, **kw)
    C = 256 if kind == "logreg" else 128
    q0 = start_positions(dt.dim, C, seed=1, scale=0.2)
    warm = gj.chees_adaptation(dt, C, dynamics=dynamics)
    (state, params), hist = warm.run(0, q0, 0.05, gj.adam(0.05), 40)
    assert math.isfinite(params["step_size"]) and params["step_size"] > 0
    assert hist[-1].adaptation_state.trajectory_length > 0.05 * 1.2
    assert all(math.isfinite(x.statistics.harmonic_mean_acceptance) for x in hist)
    dyn = {"lmc": gj.dynamic_lmc, "rmhmc": gj.dynamic_rmhmc}[dynamics]
    kern = dyn.build_kernel(params["next_random_arg_fn"], params["integration_steps_fn"])
    s, info = kern(1, state, dt, params["step_size"])
    assert s.random_generator_arg == state.random_generator_arg + 1
    assert np.isfinite(_np(s.position)).all()


def test_lmcmonge_chees_run():
    import geomjax_gb300 as gj

    dt = device_target("funnel", "mixed", D=100, metric="diag")
    C = 512
    q0 = np.ones((C, 100))
    warm = gj.lmcmonge_chees_adaptation(dt, np.ones(100), C, alpha2=1.0)
    (state, params), hist = warm.run(0, q0, 0.02, gj.adam(0.05), 100)
    assert params["alpha2"] == 1.0
    assert math.isfinite(params["step_size"]) and params["step_size"] > 0
    assert all(x.num_integration_steps >= 1 for x in hist)
    assert np.isfinite(_np(state.position)).all()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind,kw,alpha2,fix", [
    ("funnel", dict(D=7, metric="diag"), 0.5, False),
    ("funnel", dict(D=100, metric="diag"), 1.0, False),
    ("hier", dict(J=6), 0.3, True),
], ids=str)
def test_alpha2_tangent_matches_oracle_differences(kind, kw, alpha2, fix, precision):
    """gj_lmcmonge_alpha2_jvp: q_L equals the oracle's proposal position and
    ∂q_L/∂α² equals central differences of it in α² (relative step 1e-5),
    normwise max|J − FD| / max|FD| < 1e-6 in FP64.  In the mixed precision
    the arrays (and the hierarchical data) are float32: q_L to 1e-5 and the
    tangent to 1e-4."""
    from geomjax_gb300 import autodiff as AD

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, precision, **kw)
    C, h, L = 5, 0.02, 8
    q0 = start_positions(ot.dim, C, seed=3, scale=0.5)
    z, _ = normals(C, ot.dim, 4, np.float32 if precision == "mixed" else np.float64)
    im = np.linspace(0.8, 1.2, ot.dim)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
        im = im.astype(np.float32).astype(np.float64)
    qL, dq = AD.lmcmonge_alpha2_tangent(dt, q0, z, h, L, alpha2, im, fix)

    def prop(a2):
        _, oi = O_monge.kernel(ot, O_monge.init(ot, q0), z, -np.ones(C), h, im, L, alpha2=a2,
                               alpha2_fix=fix)
        return oi.proposal.position

    tol = 1e-10 if precision == "fp64" else 1e-5
    assert rel_err(_np(qL), prop(alpha2)) < tol
    e = 1e-5 * alpha2
    fd = (prop(alpha2 + e) - prop(alpha2 - e)) / (2 * e)
    err = np.max(np.abs(_np(dq) - fd)) / np.max(np.abs(fd))
    assert err < (1e-6 if precision == "fp64" else 1e-4), err


def test_lmcmonge_chees_run_updates_alpha2():
    """update_alpha: α² moves from its start by its own optimiser steps on
    the device tangent's statistic, and stays finite and positive."""
    import geomjax_gb300 as gj

    dt = device_target("funnel", "mixed", D=100, metric="diag")
    C = 512
    q0 = np.ones((C, 100))
    warm = gj.lmcmonge_chees_adaptation(dt, np.ones(100), C, alpha2=0.5, update_alpha=True)
    (state, params), hist = warm.run(0, q0, 0.02, gj.adam(0.05), 40)
    a2 = [x.adaptation_state.alpha2 for x in hist]
    assert all(math.isfinite(a) and a > 0 for a in a2)
    assert abs(a2[-1] - 0.5) > 1e-3
    assert params["alpha2"] == a2[-1]
    assert all(math.isfinite(x.statistics.alpha2_gradient) for x in hist)
