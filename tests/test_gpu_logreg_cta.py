"""The CTA-per-chain dense-Fisher logistic-regression kernels (RMHMC with
either integrator, dense LMC) against the float64 oracle, through the C ABI.

The plain FP64 form (every vector, the data and all arithmetic in float64)
must agree with the oracle to 1e-10 per step; the mixed form (float32 data,
state and per-datum arithmetic; float64 factor, solves, iterates, energies)
to 1e-5 per step over 10 steps.  Dense LMC covers the reference's
lmcmc/integrators.py:51-144 on this family at d = 25 and d = 64.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import lmc as O_lmc  # noqa: E402
from oracle import rmhmc as O_rm  # noqa: E402
from tests.helpers import device_target, normals, oracle_target, rel_err, start_positions  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-5}
IM, GL = "implicit_midpoint", "generalized_leapfrog"


def _np(t):
    return t.detach().double().cpu().numpy()


def _start(ot, C, seed, precision, scale=0.2):
    q0 = start_positions(ot.dim, C, seed=seed, scale=scale)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
    return q0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("integrator", [IM, GL])
@pytest.mark.parametrize("N,d", [(300, 9), (1000, 25), (600, 64)])
def test_rmhmc_cta_per_step(N, d, integrator, precision):
    """Positions after 1, 2, 5 and 10 steps (accept forced), the drawn
    momentum, the proposal energy, the proposal velocity and the fixed-point
    iteration counts."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=N, d=d, seed=3)
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", precision, **kw)
    C, h, L = 8, 0.05, 10
    q0 = _start(ot, C, 1, precision)
    z, _ = normals(C, d, 2, np.float32 if precision == "mixed" else np.float64)
    u = -np.ones(C)
    traj = []
    _, oinfo = O_rm.kernel(ot, O_rm.init(ot, q0), z, u, h, L, trajectory=traj,
                           integrator=integrator)
    kern = gj.rmhmc.build_kernel(logreg_path="cta", integrator=integrator)
    st0 = gj.rmhmc.init(q0, dt)
    tol = TOL[precision]
    for step in (1, 2, 5, 10):
        st, info = kern(Draws(z, u), st0, dt, h, step)
        e = rel_err(_np(st.position), traj[step - 1].position)
        assert e < tol, f"step {step}: position error {e}"
        if step == 1:
            assert rel_err(_np(info.momentum), O_rm.momentum_from_normals(ot, q0, z)) < tol
    assert rel_err(_np(info.energy), oinfo.energy) < tol * 10
    assert rel_err(_np(st.logdensity), traj[-1].logdensity) < tol * 10
    assert rel_err(_np(st.logdensity_grad), traj[-1].logdensity_grad) < tol * 10
    diff = np.abs(_np(info.fixed_point_iters) - oinfo.fixed_point_iters)
    if precision == "fp64":
        assert diff.max() <= 1, diff
    else:
        assert diff.max() <= 10 and diff.mean() < 3.0, (diff.max(), diff.mean())
    # the flipped proposal velocity −G(q_L)⁻¹p_L
    assert rel_err(_np(info.proposal.velocity), oinfo.proposal.velocity) < tol * 10


def test_rmhmc_cta_is_the_fp64_default_and_matches_thread_per_chain():
    """GJ_FP64 logistic regression runs one CTA per chain by default; at
    d <= 32 it agrees with the thread-per-chain kernel to 1e-11 over three
    transitions with real uniforms, accept decisions identical."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=200, d=8, seed=5)
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", "fp64", **kw)
    C = 32
    q0 = _start(ot, C, 4, "fp64")
    ka = gj.rmhmc.build_kernel(integrator=GL)
    kb = gj.rmhmc.build_kernel(integrator=GL, logreg_path="per_chain")
    sa = gj.rmhmc.init(q0, dt)
    sb = gj.rmhmc.init(q0, dt)
    rng = np.random.Generator(np.random.PCG64(6))
    for _ in range(3):
        z = rng.standard_normal((C, 8))
        u = rng.random(C)
        sa, ia = ka(Draws(z, u), sa, dt, 0.08, 6)
        sb, ib = kb(Draws(z, u), sb, dt, 0.08, 6)
        assert np.array_equal(_np(ia.is_accepted), _np(ib.is_accepted))
        assert rel_err(_np(sa.position), _np(sb.position)) < 1e-11
        assert rel_err(_np(ia.energy), _np(ib.energy)) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("N,d", [(300, 9), (1000, 25), (1000, 64)])
def test_lmc_cta_per_step(N, d, precision):
    """Dense-metric LMC on the logistic Fisher metric (lmcmc/integrators.py
    :51-144, lmcmc/metrics.py:75-219): positions and volume adjustments after
    1, 2, 5 and 10 steps, the drawn velocity and the proposal energy."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=N, d=d, seed=3)
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", precision, **kw)
    C, h, L = 6, 0.05, 10
    q0 = _start(ot, C, 2, precision)
    z, _ = normals(C, d, 9, np.float32 if precision == "mixed" else np.float64)
    u = -np.ones(C)
    traj = []
    _, oinfo = O_lmc.kernel(ot, O_lmc.init(ot, q0), z, u, h, L, trajectory=traj)
    kern = gj.lmc.build_kernel()
    st0 = gj.lmc.init(q0, dt)
    tol = TOL[precision]
    for step in (1, 2, 5, 10):
        st, info = kern(Draws(z, u), st0, dt, h, step)
        assert rel_err(_np(st.position), traj[step - 1].position) < tol, step
        assert rel_err(_np(st.volume_adjustment), traj[step - 1].volume_adjustment) < tol * 10
        if step == 1:
            assert rel_err(_np(info.velocity), oinfo.velocity) < tol
    assert rel_err(_np(info.energy), oinfo.energy) < tol * 10
    assert rel_err(_np(st.logdensity_grad), traj[-1].logdensity_grad) < tol * 10


@pytest.mark.parametrize("sampler", ["rmhmc", "lmc"])
def test_cta_accept_decisions_match_oracle(sampler):
    """Five chained FP64 transitions with real uniforms at a step size that
    rejects a share of the proposals: accept decisions identical to the
    oracle's, positions within 1e-10."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=1000, d=25, seed=0)
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", "fp64", **kw)
    C, h, L = 32, 0.3, 6
    q0 = _start(ot, C, 7, "fp64", scale=0.05)
    mod = gj.rmhmc if sampler == "rmhmc" else gj.lmc
    kern = mod.build_kernel()
    st = mod.init(q0, dt)
    om = O_rm if sampler == "rmhmc" else O_lmc
    so = om.init(ot, q0)
    rng = np.random.Generator(np.random.PCG64(8))
    rejected = 0
    for t in range(5):
        z = rng.standard_normal((C, 25))
        u = rng.random(C)
        so, oi = om.kernel(ot, so, z, u, h, L)
        st, info = kern(Draws(z, u), st, dt, h, L)
        acc = _np(info.is_accepted).astype(bool)
        assert np.array_equal(acc, oi.is_accepted), t
        rejected += int((~acc).sum())
        assert rel_err(_np(st.position), so.position) < 1e-10, t
    assert rejected > 0


def test_cta_rejects_unsupported_sizes():
    import geomjax_gb300 as gj
    from geomjax_gb300 import _lib as L
    from geomjax_gb300.base import Draws

    dt = device_target("logreg", "fp64", N=50, d=70)
    q0 = np.zeros((2, 70))
    kern = gj.rmhmc.build_kernel(logreg_path="cta")
    with pytest.raises(L.GeomjaxError) as ei:
        kern(Draws(np.zeros((2, 70)), np.zeros(2)), gj.rmhmc.init(q0, dt), dt, 0.05, 2)
    assert ei.value.code == L.GJ_ENOTSUP
