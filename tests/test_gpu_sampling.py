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


def test_lmcmonge_gaussian_like_moments():
    """LMC-Monge (mixed) on the hierarchical Gaussian with a single group and
    tiny observation noise is close to Gaussian in θ_1; checked against a
    long float64 run of the same kernel family for mean/variance agreement of
    μ within 2 MCSE of the difference."""
    import geomjax_gb300 as gj
    from oracle import targets as OT

    y, s = OT.make_hier_data(8, seed=4)
    C, S = 1024, 200
    means, vars_, esss = [], [], []
    for prec in ("mixed", "fp64"):
        tg = gj.hierarchical_gaussian(y, s, precision=prec)
        kern = gj.lmcmonge.build_kernel()
        dt = torch.float32 if prec == "mixed" else torch.float64
        st = gj.lmcmonge.init(torch.zeros(C, tg.dim, dtype=dt), tg)
        im = torch.ones(tg.dim, dtype=dt, device="cuda")
        gen = torch.Generator(device="cuda").manual_seed(1 if prec == "mixed" else 2)
        for _ in range(200):
            st, _ = kern(gen, st, tg, 0.2, 8, alpha2=0.1, inverse_mass_matrix=im)
        tr = torch.empty(S, C, dtype=torch.float64, device="cuda")
        for i in range(S):
            st, _ = kern(gen, st, tg, 0.2, 8, alpha2=0.1, inverse_mass_matrix=im)
            tr[i] = st.position[:, tg.J].double()  # μ
        ess = float(gj.ess(tr, chain_axis=1, sample_axis=0).item())
        means.append(float(tr.mean().item()))
        vars_.append(float(tr.var().item()))
        esss.append(ess)
    se = math.sqrt(vars_[0] / esss[0] + vars_[1] / esss[1])
    assert abs(means[0] - means[1]) < 2 * se, (means, se)
    se_v = math.sqrt(2 * vars_[0] ** 2 / esss[0] + 2 * vars_[1] ** 2 / esss[1])
    assert abs(vars_[0] - vars_[1]) < 2 * se_v, (vars_, se_v)


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
