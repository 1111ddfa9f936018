"""Sampling-level checks on the GPU: posterior moments within 2 Monte Carlo
standard errors, and the host-side adaptation loops driving the kernels."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _mcse_check(trace, true_mean, true_var, label):
    """trace [S, C]: mean and variance of one coordinate within 2 MCSE."""
    import geomjax_gb300 as gj

    x = trace.double()
    ess = float(gj.ess(x, chain_axis=1, sample_axis=0).item())
    m = float(x.mean().item())
    v = float(x.var().item())
    se_m = math.sqrt(true_var / ess)
    se_v = true_var * math.sqrt(2.0 / ess)
    assert abs(m - true_mean) < 2 * se_m, (label, m, se_m, ess)
    assert abs(v - true_var) < 2 * se_v, (label, v, se_v, ess)


def test_rmhmc_funnel_posterior_moments():
    """RMHMC with the diagonal Fisher metric on the D=2 funnel, plain FP64:
    v = θ[1] ~ N(0, 9) (mean 0, variance 9) within 2 MCSE."""
    import geomjax_gb300 as gj

    tg = gj.funnel(D=2, metric="diag", precision="fp64")
    C, S = 2048, 300
    kern = gj.rmhmc.build_kernel(max_iters=6)
    st = gj.rmhmc.init(torch.ones(C, 2, dtype=torch.float64), tg)
    gen = torch.Generator(device="cuda").manual_seed(0)
    for _ in range(100):  # burn-in
        st, _ = kern(gen, st, tg, 0.1, 10)
    tr = torch.empty(S, C, dtype=torch.float64, device="cuda")
    for s in range(S):
        st, _ = kern(gen, st, tg, 0.1, 10)
        tr[s] = st.position[:, 1]
    _mcse_check(tr, 0.0, 9.0, "v")


def test_lmcmonge_mixed_matches_fp64_posterior():
    """Equal posterior accuracy of the mixed and the plain FP64 LMC-Monge
    forms on the funnel (D = 10, α² = 1, h = 0.02, 16 steps): the mean and
    variance of v = θ[D−1] from the two forms agree within 2 Monte Carlo
    standard errors of their difference (both forms run the same burn-in, so
    what is compared is the effect of the precision, not mixing)."""
    import geomjax_gb300 as gj

    D, C, S = 10, 2048, 300
    stats = []
    for prec, seed in (("mixed", 1), ("fp64", 2)):
        tg = gj.funnel(D=D, precision=prec)
        dt = torch.float32 if prec == "mixed" else torch.float64
        kern = gj.lmcmonge.build_kernel()
        st = gj.lmcmonge.init(torch.ones(C, D, dtype=dt), tg)
        im = torch.ones(D, dtype=dt, device="cuda")
        gen = torch.Generator(device="cuda").manual_seed(seed)
        for _ in range(300):
            st, _ = kern(gen, st, tg, 0.02, 16, alpha2=1.0, inverse_mass_matrix=im)
        tr = torch.empty(S, C, dtype=torch.float64, device="cuda")
        for i in range(S):
            st, _ = kern(gen, st, tg, 0.02, 16, alpha2=1.0, inverse_mass_matrix=im)
            tr[i] = st.position[:, D - 1].double()
        ess = float(gj.ess(tr, chain_axis=1, sample_axis=0).item())
        stats.append((float(tr.mean().item()), float(tr.var().item()), ess))
    (m0, v0, e0), (m1, v1, e1) = stats
    se = math.sqrt(v0 / e0 + v1 / e1)
    assert abs(m0 - m1) < 2 * se, stats

    se_v = math.sqrt(2 * v0 ** 2 / e0 + 2 * v1 ** 2 / e1)
    assert abs(v0 - v1) < 2 * se_v, stats


def test_lmcmonge_mixed_matches_fp64_posterior_d100():
    """Equal posterior accuracy at the LMC-Monge benchmark's size (funnel
    D = 100, α² = 1, h = 0.02, 16 steps): 2048 chains started at exact draws
    of the funnel run 200 transitions in the mixed form (warp per chain,
    float32 state) and in the plain FP64 form (float64 throughout) with the
    same draws.  Every coordinate's mean and variance agree within 2 Monte
    Carlo standard errors of the FP64 run.  The chains are coupled only
    until a decision differs (deep in the funnel's neck the trajectories are
    chaotic, so a float32 rounding can flip one); the chain then follows its
    own path, so the pairwise decision agreement is a coupling statistic,
    checked loosely here (the per-transition agreement from a common state is
    test_accept_agreement_monge_funnel100's, >= 99.9 %)."""
    import geomjax_gb300 as gj

    D, C, S = 100, 2048, 200
    g = torch.Generator(device="cuda").manual_seed(11)
    v = 3.0 * torch.randn(C, 1, generator=g, device="cuda", dtype=torch.float64)
    x = torch.randn(C, D - 1, generator=g, device="cuda", dtype=torch.float64) * torch.exp(0.5 * v)
    q0 = torch.cat([x, v], dim=1).float().double()
    arms = {}
    for prec in ("mixed", "fp64"):
        tg = gj.funnel(D=D, precision=prec)
        dt = torch.float32 if prec == "mixed" else torch.float64
        kern = gj.lmcmonge.build_kernel()
        st = gj.lmcmonge.init(q0.to(dt), tg)
        info = kern.new_info(C, D, tg, "cuda")
        im = torch.ones(D, dtype=dt, device="cuda")
        gz = torch.Generator(device="cuda").manual_seed(12)
        tr = torch.empty(S, C, D, dtype=torch.float64, device="cuda")
        acc = torch.empty(S, C, dtype=torch.uint8, device="cuda")
        for i in range(S):
            z = torch.randn(C, D, generator=gz, device="cuda").to(dt)
            u = torch.rand(C, generator=gz, device="cuda", dtype=torch.float64)
            kern.step_inplace(tg, st, z, u, info, 0.02, 16, alpha2=1.0, inverse_mass=im)
            tr[i] = st.position.double()
            acc[i] = info["is_accepted"]
        arms[prec] = (tr, acc)
    (tm, am), (tp, ap) = arms["mixed"], arms["fp64"]
    ess = gj.ess(tp, chain_axis=1, sample_axis=0)
    a, b = tm.reshape(-1, D), tp.reshape(-1, D)
    mb, vb = b.mean(0), b.var(0)
    se_m = torch.sqrt(vb / ess)
    se_v = torch.sqrt(((b - mb) ** 4).mean(0) - vb * vb) / torch.sqrt(ess)
    dm = ((a.mean(0) - mb).abs() / se_m).cpu().numpy()
    dv = ((a.var(0) - vb).abs() / se_v).cpu().numpy()
    assert np.all(dm < 2.0), dm.max()
    assert np.all(dv < 2.0), dv.max()
    assert float((am == ap).double().mean()) >= 0.95


def test_window_adaptation_lmcmonge():
    """window_adaptation drives the LMC-Monge kernel; the adapted step size
    gives a mean acceptance near the 0.8 target and a positive inverse mass."""
    import geomjax_gb300 as gj
    from geomjax_gb300.adaptation import window_adaptation

    tg = gj.funnel(D=10, precision="mixed")
    wa = window_adaptation(gj.lmcmonge, tg, initial_step_size=0.05, target_acceptance_rate=0.8,
                           num_integration_steps=8, alpha2=1.0)
    (state, params), infos = wa.run(3, torch.zeros(512, 10), num_steps=300)
    assert params["step_size"] > 0 and torch.all(params["inverse_mass_matrix"] > 0)
    kern = gj.lmcmonge.build_kernel()
    gen = torch.Generator(device="cuda").manual_seed(9)
    acc = []
    for _ in range(30):
        state, info = kern(gen, state, tg, params["step_size"], 8, alpha2=1.0,
                           inverse_mass_matrix=params["inverse_mass_matrix"])
        acc.append(float(info.acceptance_rate.mean().item()))
    assert 0.6 < np.mean(acc) < 0.97, np.mean(acc)


def test_step_size_adaptation_rmhmc_logreg():
    """step_size_adaptation drives the batched dense-Fisher RMHMC kernel."""
    import geomjax_gb300 as gj
    from geomjax_gb300.adaptation import step_size_adaptation
    from geomjax_gb300.data import logreg_data

    X, y = logreg_data(300, 6, seed=2)
    tg = gj.logistic_regression(X, y, precision="mixed")
    ssa = step_size_adaptation(gj.rmhmc, tg, initial_step_size=0.5, target_acceptance_rate=0.8,
                               num_integration_steps=4)
    (state, params), infos = ssa.run(5, torch.zeros(256, 6), num_steps=60)
    assert 0.02 < params["step_size"] < 2.0
    assert abs(np.mean(infos[-20:]) - 0.8) < 0.15


@pytest.mark.parametrize("alg", ["nutsrmhmc", "nutslmcmonge"])
def test_window_adaptation_nuts(alg):
    """window_adaptation drives the NUTS samplers (the Monge one adapts its
    inverse mass too); the adapted step size keeps NUTS's mean acceptance
    statistic near the target."""
    import geomjax_gb300 as gj
    from geomjax_gb300.adaptation import window_adaptation

    algorithm = getattr(gj, alg)
    if alg == "nutsrmhmc":
        tg = gj.funnel(D=2, precision="fp64")
        extra = dict(max_num_doublings=6)
    else:
        tg = gj.funnel(D=10, precision="mixed")
        extra = dict(max_num_doublings=6, alpha2=1.0)
    wa = window_adaptation(algorithm, tg, initial_step_size=0.1, target_acceptance_rate=0.8,
                           **extra)
    (state, params), infos = wa.run(4, torch.zeros(256, tg.dim), num_steps=150)
    assert params["step_size"] > 0 and params["max_num_doublings"] == 6
    if alg == "nutslmcmonge":
        assert torch.all(params["inverse_mass_matrix"] > 0)
    assert 0.55 < np.mean(infos[-40:]) < 0.97, np.mean(infos[-40:])
