"""Parity of the batched mixed-precision RMHMC path at the benchmark's own
configuration: Bayesian logistic regression on the seeded data the benchmark
uses (N = 1000, d = 25), 4096 chains on the device, with the float64 oracle
run on a fixed sample of 64 of them (rmhmc/rmhmc.py:131-174,
rmhmc/integrators.py:92-156 and the generalized leapfrog).

* per-step positions within 1e-5 over 10 steps, both integrators;
* accept decisions agree on >= 99.9 % of 20 transitions with real uniforms,
  at step sizes where a share of the proposals is rejected;
* posterior means and variances of every coordinate within 2 Monte Carlo
  standard errors of a float64 run (the plain CTA-per-chain form) fed the
  same draws;
* one posterior at the uneven batch's largest size, N = 5000, d = 128.

Chains start from draws of the posterior's Laplace approximation, so every
check runs in the typical set rather than in a burn-in transient.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import rmhmc as O_rm  # noqa: E402
from oracle import targets as OT  # noqa: E402
from tests.helpers import laplace_draws, rel_err  # noqa: E402

pytestmark = pytest.mark.gpu

IM, GL = "implicit_midpoint", "generalized_leapfrog"
C = 4096
SAMPLE = np.arange(0, C, C // 64)  # 64 chains spread over the batch


def _np(t):
    return t.detach().double().cpu().numpy()


def _targets(N=1000, d=25, precision="mixed"):
    import geomjax_gb300 as gj
    from geomjax_gb300.data import logreg_data

    X, y = logreg_data(N, d, seed=0)
    return OT.LogisticRegression(X, y), gj.logistic_regression(X, y, precision=precision)


def _f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("integrator", [GL, IM])
def test_headline_per_step(integrator):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot, dt = _targets()
    q0 = _f32(laplace_draws(ot, C, seed=1))
    rng = np.random.Generator(np.random.PCG64(2))
    z = _f32(rng.standard_normal((C, 25)))
    u = -np.ones(C)  # accept forced: the proposal itself is compared
    h, L = 0.05, 10
    traj = []
    _, oinfo = O_rm.kernel(ot, O_rm.init(ot, q0[SAMPLE]), z[SAMPLE], u[SAMPLE], h, L,
                           trajectory=traj, integrator=integrator)
    kern = gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=integrator)
    st0 = gj.rmhmc.init(q0, dt)
    for step in range(1, L + 1):
        st, info = kern(Draws(z, u), st0, dt, h, step)
        e = rel_err(_np(st.position)[SAMPLE], traj[step - 1].position)
        assert e < 1e-5, f"step {step}: position error {e}"
    assert rel_err(_np(info.energy)[SAMPLE], oinfo.energy) < 1e-4
    assert rel_err(_np(st.logdensity_grad)[SAMPLE], traj[-1].logdensity_grad) < 1e-4
    diff = np.abs(_np(info.fixed_point_iters)[SAMPLE] - oinfo.fixed_point_iters)
    assert diff.max() <= 10 and diff.mean() < 2.5, (diff.max(), diff.mean())


@pytest.mark.parametrize("integrator,h", [(GL, 0.8), (IM, 1.3)])
def test_headline_accept_agreement(integrator, h):
    """Each transition starts the oracle from the device's current state of the
    sampled chains; 20 transitions of 8 steps with real uniforms."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot, dt = _targets()
    kern = gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=integrator)
    st = gj.rmhmc.init(_f32(laplace_draws(ot, C, seed=3)), dt)
    rng = np.random.Generator(np.random.PCG64(4))
    agree = total = rejected = 0
    for t in range(20):
        z = _f32(rng.standard_normal((C, 25)))
        u = rng.random(C)
        so = O_rm.RMHMCState(_np(st.position)[SAMPLE], _np(st.logdensity)[SAMPLE],
                             _np(st.logdensity_grad)[SAMPLE])
        _, oi = O_rm.kernel(ot, so, z[SAMPLE], u[SAMPLE], h, 8, integrator=integrator)
        st, info = kern(Draws(z, u), st, dt, h, 8)
        a = _np(info.is_accepted).astype(bool)[SAMPLE]
        agree += int(np.sum(a == oi.is_accepted))
        total += len(SAMPLE)
        rejected += int(np.sum(~oi.is_accepted))
    assert rejected >= 0.1 * total, rejected  # the decisions are not all "accept"
    assert agree / total >= 0.999, (agree, total)


def test_headline_posterior_moments_within_2_mcse():
    """The mixed batched path (4096 chains) and the plain FP64 form (one CTA
    per chain, float64 throughout; its first 512 chains) run 100 transitions
    from the same positions with the same draws.  Every coordinate's posterior
    mean and variance over those 512 chains agree within 2 Monte Carlo
    standard errors of the float64 run (ESS of diagnostics.py:78-209)."""
    import geomjax_gb300 as gj

    ot, dt = _targets()
    pt = _targets(precision="fp64")[1]
    Cp, T, h, L = 512, 100, 0.05, 8
    q0 = _f32(laplace_draws(ot, C, seed=5))
    km = gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=GL)
    kp = gj.rmhmc.build_kernel(integrator=GL)  # GJ_FP64 default: one CTA per chain
    sm = gj.rmhmc.init(q0, dt)
    sp = gj.rmhmc.init(q0[:Cp], pt)
    im = km.new_info(C, 25, dt, dt.device)
    ip = kp.new_info(Cp, 25, pt, pt.device)
    g = torch.Generator(device="cuda").manual_seed(6)
    tm = torch.empty(T, Cp, 25, dtype=torch.float64, device="cuda")
    tp = torch.empty_like(tm)
    agree = 0
    for t in range(T):
        z = torch.randn(C, 25, generator=g, device="cuda")
        u = torch.rand(C, generator=g, device="cuda", dtype=torch.float64)
        km.step_inplace(dt, sm, z, u, im, h, L)
        kp.step_inplace(pt, sp, z[:Cp].double(), u[:Cp], ip, h, L)
        tm[t] = sm.position[:Cp].double()
        tp[t] = sp.position
        agree += int((im["is_accepted"][:Cp] == ip["is_accepted"]).sum())
    ess = gj.effective_sample_size(tp, chain_axis=1, sample_axis=0)
    a, b = tm.reshape(-1, 25), tp.reshape(-1, 25)
    mb, vb = b.mean(0), b.var(0)
    se_mean = torch.sqrt(vb / ess)
    se_var = torch.sqrt(((b - mb) ** 4).mean(0) - vb * vb) / torch.sqrt(ess)
    dm = ((a.mean(0) - mb).abs() / se_mean).cpu().numpy()
    dv = ((a.var(0) - vb).abs() / se_var).cpu().numpy()
    assert np.all(dm < 2.0), dm
    assert np.all(dv < 2.0), dv
    assert agree / (T * Cp) >= 0.999


def test_c4_largest_posterior_per_step():
    """One posterior at the uneven batch's upper sizes (N = 5000, d = 128),
    64 chains on the batched path, 16 of them through the oracle: per-step
    positions over 10 steps within 1e-5 (generalized leapfrog)."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot, dt = _targets(N=5000, d=128)
    Cb = 64
    S = np.arange(0, Cb, 4)
    q0 = _f32(laplace_draws(ot, Cb, seed=7))
    rng = np.random.Generator(np.random.PCG64(8))
    z = _f32(rng.standard_normal((Cb, 128)))
    u = -np.ones(Cb)
    h, L = 0.05, 10
    traj = []
    O_rm.kernel(ot, O_rm.init(ot, q0[S]), z[S], u[S], h, L, trajectory=traj, integrator=GL)
    kern = gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=GL)
    st0 = gj.rmhmc.init(q0, dt)
    for step in (1, 2, 5, 10):
        st, _ = kern(Draws(z, u), st0, dt, h, step)
        e = rel_err(_np(st.position)[S], traj[step - 1].position)
        assert e < 1e-5, f"step {step}: position error {e}"


@pytest.mark.parametrize("N,d,path,bound", [
    (1000, 25, "tcgen05", 3e-5), (1000, 25, "simt", 3e-5), (1000, 25, "cta", 1e-6),
    (2000, 64, "cta", 1e-5)])
def test_momentum_draw_accuracy_by_path(N, d, path, bound):
    """The drawn momentum chol(G)·z against the oracle's, by implementation:
    the batched paths carry their FP32 Gram's rounding through the factor
    (≈ 1e-5 at d = 25, growing with d); the CTA form sums its Gram's 16-row
    tiles in float64 (≈ 3e-7 at d = 25, 2e-6 at d = 64)."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot, dt = _targets(N=N, d=d)
    Cb = 64
    S = np.arange(0, Cb, 8)
    q0 = _f32(laplace_draws(ot, Cb, seed=1))
    z = _f32(np.random.default_rng(2).standard_normal((Cb, d)))
    kern = gj.rmhmc.build_kernel(logreg_path=path, integrator=GL, loop="host")
    _, info = kern(Draws(z, -np.ones(Cb)), gj.rmhmc.init(q0, dt), dt, 0.05, 1)
    ref = O_rm.momentum_from_normals(ot, q0[S], z[S])
    assert rel_err(_np(info.momentum)[S], ref) < bound


@pytest.mark.parametrize("N,d", [(1000, 25), (300, 9), (400, 32), (100, 8)])
def test_fused_r2x_matches_stored_r2(N, d):
    """The momentum evaluations' r₂·X formed inside the S = U·Xᵀ GEMM (r₂
    written as three BF16 planes into the kernel's freed operand ring and
    contracted against the Xᵀ boxes on the tensor cores, one partial gradient
    per N tile, added in tile order) against r₂ stored in global memory and
    contracted by a second GEMM: both within 1e-5 of the oracle per step over
    10 generalized-leapfrog steps, and within 2e-6 of each other."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot, dt = _targets(N=N, d=d)
    Cb = 256
    S = np.arange(0, Cb, 16)
    q0 = _f32(laplace_draws(ot, Cb, seed=11))
    z = _f32(np.random.default_rng(12).standard_normal((Cb, d)))
    u = -np.ones(Cb)
    h, L = 0.05, 10
    traj = []
    O_rm.kernel(ot, O_rm.init(ot, q0[S]), z[S], u[S], h, L, trajectory=traj, integrator=GL)
    kf = gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=GL, fuse_r2x=True)
    ks = gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=GL, fuse_r2x=False)
    st0 = gj.rmhmc.init(q0, dt)
    for step in (1, 5, 10):
        sf, inf_f = kf(Draws(z, u), st0, dt, h, step)
        ss, inf_s = ks(Draws(z, u), st0, dt, h, step)
        pf, ps = _np(sf.position), _np(ss.position)
        ef, es = (rel_err(pf[S], traj[step - 1].position),
                  rel_err(ps[S], traj[step - 1].position))
        assert rel_err(pf, ps) < 2e-6, (step, rel_err(pf, ps), ef, es)
        assert ef < 1e-5 and es < 1e-5, (step, ef, es)
    diff = np.abs(_np(inf_f.fixed_point_iters) - _np(inf_s.fixed_point_iters))
    assert diff.mean() < 1.0, diff.mean()
