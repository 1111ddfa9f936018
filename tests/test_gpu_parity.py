"""GPU parity of the CUDA kernels against the float64 oracle, through the
C ABI (via the geomjax_gb300 host API, which calls it with ctypes).

Error measure: e = max |gpu − oracle| / (1 + |oracle|) per element.
Tolerances: the plain FP64 form 1e-12 (1e-10 where a fixed-point solve or
a long data sum sits in between); the mixed form (FP32 state, BF16-split
contractions) 1e-5 per step over 10 steps, as the parity contract states.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import lmc as O_lmc  # noqa: E402
from oracle import lmcmonge as O_monge  # noqa: E402
from oracle import rmhmc as O_rm  # noqa: E402
from tests.helpers import device_target, normals, oracle_target, rel_err, start_positions  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "mixed": 1e-5}

OP_CASES = [
    ("funnel", dict(D=2, metric="diag")),
    ("funnel", dict(D=100, metric="diag")),
    ("funnel", dict(D=5, metric="pullback")),
    ("logreg", dict(N=64, d=6)),
    ("hier", dict(J=6)),
]


def _np(t):
    return t.detach().double().cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind,kw", OP_CASES, ids=lambda x: str(x))
def test_operators(kind, kw, precision):
    ot = oracle_target(kind, **kw)
    dt = device_target(kind, precision, **kw)
    q = start_positions(ot.dim, 7, seed=3)
    if precision == "mixed":
        q = q.astype(np.float32).astype(np.float64)
    u = start_positions(ot.dim, 7, seed=4)
    if precision == "mixed":
        u = u.astype(np.float32).astype(np.float64)
    ld, g = dt.logdensity_and_grad(q)
    tol = 1e-12 if precision == "fp64" else 2e-5
    assert rel_err(_np(ld), ot.logdensity(q)) < tol * 10
    assert rel_err(_np(g), ot.grad(q)) < tol
    assert rel_err(_np(dt.hvp(q, u)), ot.hvp(q, u)) < tol
    if ot.dim <= 32:
        assert rel_err(_np(dt.metric_fn(q)), ot.metric(q)) < tol


def _rm_case(kind, kw, precision, integrator, h, L, max_iters, C=6, seed=0):
    import geomjax_gb300 as gj

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, precision, **kw)
    q0 = start_positions(ot.dim, C, seed=seed, scale=0.3)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
    z, _ = normals(C, ot.dim, seed + 1, np.float32 if precision == "mixed" else np.float64)
    u = -np.ones(C)  # u < p_accept always holds: the proposal itself is compared
    kern = gj.rmhmc.build_kernel(integrator=integrator, max_iters=max_iters)
    st0 = gj.rmhmc.init(q0, dt)
    so = O_rm.init(ot, q0)
    traj = []
    _, oinfo = O_rm.kernel(ot, so, z, u, h, L, integrator=integrator, max_iters=max_iters,
                           trajectory=traj)
    return gj, ot, dt, kern, st0, q0, z, u, traj, oinfo


@pytest.mark.parametrize("integrator", ["implicit_midpoint", "generalized_leapfrog"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind,kw", [
    ("funnel", dict(D=2, metric="diag")),
    ("funnel", dict(D=4, metric="pullback")),
    ("hier", dict(J=5)),
    ("logreg", dict(N=40, d=4)),
], ids=lambda x: str(x))
def test_rmhmc_per_step(kind, kw, precision, integrator):
    """Positions after every one of 10 steps (one transition per trajectory
    length, accept forced with u = 0), the drawn momentum and the final energy."""
    h, L, mi = 0.05, 10, 100
    gj, ot, dt, kern, st0, q0, z, u, traj, oinfo = _rm_case(kind, kw, precision, integrator, h, L,
                                                             mi)
    from geomjax_gb300.base import Draws

    opts = dict(logreg_path="per_chain") if kind == "logreg" else {}
    kern = gj.rmhmc.build_kernel(integrator=integrator, max_iters=mi, **opts)
    tol = TOL[precision]
    for step in range(1, L + 1):
        st, info = kern(Draws(z, u), st0, dt, h, step)
        e = rel_err(_np(st.position), traj[step - 1].position)
        assert e < tol, f"step {step}: position error {e}"
        if step == 1:
            assert rel_err(_np(info.momentum), O_rm.momentum_from_normals(ot, q0, z)) < tol
    assert rel_err(_np(info.energy), oinfo.energy) < tol * 10
    assert rel_err(_np(st.logdensity), traj[-1].logdensity) < tol * 10
    assert rel_err(_np(st.logdensity_grad), traj[-1].logdensity_grad) < tol * 10


def test_plain_fp64_funnel_config():
    """The plain FP64 configuration: funnel D=2, diagonal Fisher metric,
    h = 0.1, 10 steps, 6 fixed-point iterations, 4 chains, 20 transitions
    from ones(2) (examples/funnel/main.py:69), seeded host draws; positions,
    log densities and accept decisions agree with the oracle to 1e-12."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target("funnel", D=2, metric="diag")
    dt = device_target("funnel", "fp64", D=2, metric="diag")
    C = 4
    q0 = np.ones((C, 2))
    kern = gj.rmhmc.build_kernel(max_iters=6)
    st = gj.rmhmc.init(q0, dt)
    so = O_rm.init(ot, q0)
    rng = np.random.Generator(np.random.PCG64(0))
    for t in range(20):
        z = rng.standard_normal((C, 2))
        u = rng.random(C)
        so, oi = O_rm.kernel(ot, so, z, u, 0.1, 10, max_iters=6)
        st, info = kern(Draws(z, u), st, dt, 0.1, 10)
        assert np.array_equal(_np(info.is_accepted).astype(bool), oi.is_accepted)
        assert rel_err(_np(st.position), so.position) < 1e-12, t
        assert rel_err(_np(st.logdensity), so.logdensity) < 1e-12
        assert rel_err(_np(info.acceptance_rate), oi.acceptance_rate) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind,kw", [
    ("funnel", dict(D=3, metric="diag")),
    ("funnel", dict(D=4, metric="pullback")),
    ("hier", dict(J=4)),
], ids=lambda x: str(x))
def test_lmc_dense_per_step(kind, kw, precision):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, precision, **kw)
    C, h, L = 5, 0.05, 10
    q0 = start_positions(ot.dim, C, seed=2, scale=0.3)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
    z, _ = normals(C, ot.dim, 9, np.float32 if precision == "mixed" else np.float64)
    u = -np.ones(C)
    traj = []
    _, oinfo = O_lmc.kernel(ot, O_lmc.init(ot, q0), z, u, h, L, trajectory=traj)
    kern = gj.lmc.build_kernel()
    st0 = gj.lmc.init(q0, dt)
    for step in range(1, L + 1):
        st, info = kern(Draws(z, u), st0, dt, h, step)
        assert rel_err(_np(st.position), traj[step - 1].position) < TOL[precision], step
        assert rel_err(_np(st.volume_adjustment), traj[step - 1].volume_adjustment) < TOL[precision] * 10
    assert rel_err(_np(info.energy), oinfo.energy) < TOL[precision] * 10


@pytest.mark.parametrize("alpha2_fix", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("kind,kw,alpha2", [
    ("funnel", dict(D=100, metric="diag"), 1.0),
    ("funnel", dict(D=7, metric="diag"), 0.3),
    ("hier", dict(J=30), 0.5),
], ids=lambda x: str(x))
def test_lmcmonge_per_step(kind, kw, alpha2, precision, alpha2_fix):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, precision, **kw)
    C, h, L = 9, 0.02, 10
    q0 = start_positions(ot.dim, C, seed=5, scale=0.5)
    if precision == "mixed":
        q0 = q0.astype(np.float32).astype(np.float64)
    z, _ = normals(C, ot.dim, 11, np.float32 if precision == "mixed" else np.float64)
    u = -np.ones(C)
    im = np.linspace(0.8, 1.2, ot.dim)
    if precision == "mixed":
        im = im.astype(np.float32).astype(np.float64)
    traj = []
    _, oinfo = O_monge.kernel(ot, O_monge.init(ot, q0), z, u, h, im, L, alpha2=alpha2,
                              alpha2_fix=alpha2_fix, trajectory=traj)
    kern = gj.lmcmonge.build_kernel(alpha2_fix=alpha2_fix)
    st0 = gj.lmcmonge.init(q0, dt)
    imt = torch.as_tensor(im, dtype=dt.dtype, device="cuda")
    for step in range(1, L + 1):
        st, info = kern(Draws(z, u), st0, dt, h, step, alpha2=alpha2, inverse_mass_matrix=imt)
        assert rel_err(_np(st.position), traj[step - 1].position) < TOL[precision], step
    assert rel_err(_np(info.velocity), traj and O_monge.velocity_dense(
        alpha2, im, im * ot.grad(q0) / np.sqrt(O_monge.normalizing_constant(alpha2, im, ot.grad(q0)))[:, None], z)) < TOL[precision]
    assert rel_err(_np(info.energy), oinfo.energy) < TOL[precision] * 10
    assert rel_err(_np(st.volume_adjustment), traj[-1].volume_adjustment) < TOL[precision] * 10


@pytest.mark.parametrize("kind,kw", [("funnel", dict(D=100, metric="diag")), ("hier", dict(J=30))],
                         ids=str)
def test_lmcmonge_warp_fp64_matches_thread_per_chain(kind, kw):
    """The plain FP64 LMC-Monge form runs one warp per chain by default; it
    agrees with the thread-per-chain FP64 kernel to 1e-11 over three chained
    transitions with real uniforms, accept decisions identical."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target(kind, **kw)
    dt = device_target(kind, "fp64", **kw)
    C = 96
    q0 = start_positions(ot.dim, C, seed=3, scale=0.5)
    ka = gj.lmcmonge.build_kernel()
    kb = gj.lmcmonge.build_kernel(warp=False)
    sa, sb = gj.lmcmonge.init(q0, dt), gj.lmcmonge.init(q0, dt)
    im = torch.ones(ot.dim, dtype=torch.float64, device="cuda")
    rng = np.random.Generator(np.random.PCG64(4))
    for _ in range(3):
        z = rng.standard_normal((C, ot.dim))
        u = rng.random(C)
        sa, ia = ka(Draws(z, u), sa, dt, 0.02, 16, alpha2=1.0, inverse_mass_matrix=im)
        sb, ib = kb(Draws(z, u), sb, dt, 0.02, 16, alpha2=1.0, inverse_mass_matrix=im)
        assert np.array_equal(_np(ia.is_accepted), _np(ib.is_accepted))
        assert rel_err(_np(sa.position), _np(sb.position)) < 1e-11
        assert rel_err(_np(sa.volume_adjustment), _np(sb.volume_adjustment)) < 1e-11


def test_identity_metric_structural_pin():
    """tests/test_samplers.py:21-57 on the device: RMHMC with G = I and dense
    LMC with G = I give the HMC velocity-Verlet proposal (rtol 1e-4)."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws
    from oracle import hmc as O_hmc

    base = oracle_target("funnel", D=2)
    dt = device_target("funnel", "fp64", D=2, metric="identity")
    C = 16
    rng = np.random.default_rng(42)
    z = rng.standard_normal((C, 2))
    u = rng.random(C)
    q0 = np.zeros((C, 2))
    q_hmc, _ = O_hmc.kernel(base, q0, z, u, 1e-2, 10)
    s1, _ = gj.rmhmc.build_kernel()(Draws(z, u), gj.rmhmc.init(q0, dt), dt, 1e-2, 10)
    s3, _ = gj.lmc.build_kernel()(Draws(z, u), gj.lmc.init(q0, dt), dt, 1e-2, 10)
    np.testing.assert_allclose(_np(s1.position), q_hmc, rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(_np(s3.position), q_hmc, rtol=1e-4, atol=1e-7)


def test_accept_agreement_monge_funnel100():
    """Accept decisions of the mixed LMC-Monge kernel agree with the FP64
    oracle on >= 99.9% of transitions (each transition starts both from the
    device state; funnel D=100, α² = 1, h = 0.02, 16 steps)."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    ot = oracle_target("funnel", D=100)
    dt = device_target("funnel", "mixed", D=100)
    C, T = 256, 8
    kern = gj.lmcmonge.build_kernel()
    st = gj.lmcmonge.init(np.ones((C, 100)) * 0.5, dt)
    im = torch.ones(100, dtype=torch.float32, device="cuda")
    rng = np.random.Generator(np.random.PCG64(7))
    agree = total = 0
    for t in range(T):
        z = rng.standard_normal((C, 100)).astype(np.float32).astype(np.float64)
        u = rng.random(C)
        so = O_monge.LMCState(_np(st.position), _np(st.logdensity), _np(st.logdensity_grad),
                              _np(st.volume_adjustment))
        _, oi = O_monge.kernel(ot, so, z, u, 0.02, np.ones(100), 16, alpha2=1.0)
        st, info = kern(Draws(z, u), st, dt, 0.02, 16, alpha2=1.0, inverse_mass_matrix=im)
        a = _np(info.is_accepted).astype(bool)
        agree += int(np.sum(a == oi.is_accepted))
        total += C
    assert agree / total >= 0.999


IM, GL = "implicit_midpoint", "generalized_leapfrog"


@pytest.mark.parametrize("path,loop,chol,d,C,integrator", [
    ("simt", "host", "fp64", 9, 160, IM), ("tcgen05", "host", "fp64", 9, 160, IM),
    ("tcgen05", "graph", "fp64", 9, 160, IM), ("simt", "graph", "fp64", 9, 160, IM),
    ("tcgen05", "graph", "fp32", 9, 160, IM),
    # 8 chains share a warp in the factorisation at d = 9; at d = 40 two do,
    # and 37 chains leave a ragged last warp
    ("tcgen05", "graph", "fp64", 40, 37, IM), ("tcgen05", "host", "fp32", 40, 37, IM),
    # the generalized leapfrog: momentum solves on the stored factor and w,
    # position solves, the explicit final momentum
    ("tcgen05", "graph", "fp64", 9, 160, GL), ("tcgen05", "host", "fp64", 9, 160, GL),
    ("simt", "host", "fp64", 9, 160, GL), ("tcgen05", "graph", "fp64", 40, 37, GL),
    ("tcgen05", "graph", "fp32", 9, 160, GL),
    # a CTA per chain in the factorisation: 4 warps at d = 100 (FP64 and
    # FP32), 8 at d = 120 (FP64), with L⁻¹ in the pair table's place
    ("tcgen05", "graph", "fp64", 100, 16, GL), ("tcgen05", "host", "fp32", 100, 16, GL),
    ("tcgen05", "graph", "fp64", 120, 16, GL)])
def test_logreg_batched_per_step(path, loop, chol, d, C, integrator):
    """The batched dense-Fisher path (split-BF16 contractions, FP64 fixed-point
    iterates, FP64 or FP32 factorisation, host-driven loop or one CUDA-graph
    launch, either integrator) against the oracle: per-step positions over
    10 steps within 1e-5 (1e-4 for the FP32 factorisation at d >= 64, whose
    rounding grows with d)."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=300 if d < 32 else (500 if d < 64 else 1500), d=d, seed=3)
    tol = 1e-4 if (chol == "fp32" and d >= 64) else 1e-5
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", "mixed", **kw)
    h, L = 0.05, 10
    q0 = start_positions(ot.dim, C, seed=1, scale=0.2).astype(np.float32).astype(np.float64)
    z, _ = normals(C, ot.dim, 2, np.float32)
    u = -np.ones(C)
    traj = []
    _, oinfo = O_rm.kernel(ot, O_rm.init(ot, q0), z, u, h, L, trajectory=traj,
                           integrator=integrator)
    kern = gj.rmhmc.build_kernel(logreg_path=path, loop=loop, cholesky=chol,
                                 integrator=integrator)
    st0 = gj.rmhmc.init(q0, dt)
    for step in (1, 2, 5, 10):
        st, info = kern(Draws(z, u), st0, dt, h, step)
        e = rel_err(_np(st.position), traj[step - 1].position)
        assert e < tol, f"step {step}: {e}"
    assert rel_err(_np(info.energy), oinfo.energy) < 10 * tol
    # iteration counts over the 10 solves agree up to solves whose norm lands
    # next to the tolerance (FP32-level rounding of the map, more of it at
    # larger d); no solve may run away towards max_iters
    diff = np.abs(_np(info.fixed_point_iters) - oinfo.fixed_point_iters)
    assert diff.max() <= 10 and diff.mean() < (2.5 if d < 32 else 5.0), (diff.max(), diff.mean())


@pytest.mark.parametrize("ksplit", [1, 2, 3])
def test_logreg_batched_gradient_ksplit(ksplit):
    """The gradient contraction [r1; r2]·X with its K blocks split over 1, 2
    or 3 CTAs per output tile (partial products added in slice order by the
    consumers): per-step positions of the generalized leapfrog against the
    oracle within 1e-5, as unsplit."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=300, d=9, seed=3)  # 5 K blocks of 64 observations
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", "mixed", **kw)
    C, h, L = 160, 0.05, 10
    q0 = start_positions(ot.dim, C, seed=1, scale=0.2).astype(np.float32).astype(np.float64)
    z, _ = normals(C, ot.dim, 2, np.float32)
    u = -np.ones(C)
    traj = []
    O_rm.kernel(ot, O_rm.init(ot, q0), z, u, h, L, trajectory=traj, integrator=GL)
    kern = gj.rmhmc.build_kernel(logreg_path="tcgen05", loop="graph", integrator=GL,
                                 gemm_ksplit=ksplit)
    st0 = gj.rmhmc.init(q0, dt)
    for step in (1, 5, 10):
        st, _ = kern(Draws(z, u), st0, dt, h, step)
        e = rel_err(_np(st.position), traj[step - 1].position)
        assert e < 1e-5, f"step {step}: {e}"
        assert rel_err(_np(st.logdensity_grad), traj[step - 1].logdensity_grad) < 1e-4


def test_logreg_batched_accept_and_graph_reuse():
    """Several transitions through one graph (the captured graph is reused and
    the step size changes between calls) agree with the oracle transition by
    transition, accept decisions included."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=200, d=7, seed=5)
    ot = oracle_target("logreg", **kw)
    dt = device_target("logreg", "mixed", **kw)
    C = 128
    q0 = start_positions(ot.dim, C, seed=3, scale=0.2).astype(np.float32).astype(np.float64)
    kern = gj.rmhmc.build_kernel(logreg_path="tcgen05", loop="graph")
    st = gj.rmhmc.init(q0, dt)
    rng = np.random.Generator(np.random.PCG64(11))
    agree = total = 0
    for t, h in enumerate([0.05, 0.04, 0.06, 0.05]):
        z = rng.standard_normal((C, ot.dim)).astype(np.float32).astype(np.float64)
        u = rng.random(C)
        so = O_rm.RMHMCState(_np(st.position), _np(st.logdensity), _np(st.logdensity_grad))
        so1, oi = O_rm.kernel(ot, so, z, u, h, 6)
        st, info = kern(Draws(z, u), st, dt, h, 6)
        a = _np(info.is_accepted).astype(bool)
        agree += int(np.sum(a == oi.is_accepted))
        total += C
        same = a == oi.is_accepted
        assert rel_err(_np(st.position)[same], so1.position[same]) < 1e-5
        assert rel_err(_np(st.logdensity)[same], so1.logdensity[same]) < 1e-4
    assert agree / total >= 0.99


@pytest.mark.parametrize("groups,N,d,C", [(2, 300, 9, 301), (3, 300, 9, 301),
                                         (2, 700, 25, 1024)])
def test_logreg_batched_chain_groups_bitwise(groups, N, d, C):
    """Chains are independent: splitting them into groups whose graphs run on
    concurrent streams gives bit-identical transitions (positions, log
    densities, accept decisions, energies, fixed-point counts).  At N = 700,
    d = 25 and 1024 chains the gradient contraction is split in K, the same
    way for every group count."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=N, d=d, seed=3)
    dt = device_target("logreg", "mixed", **kw)
    q0 = start_positions(dt.dim, C, seed=1, scale=0.2).astype(np.float32).astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(5))
    out = {}
    for g in (1, groups):
        kern = gj.rmhmc.build_kernel(loop="graph", chain_groups=g)
        st = gj.rmhmc.init(q0, dt)
        rng = np.random.Generator(np.random.PCG64(5))
        rec = []
        for h in (0.05, 0.04):
            z = rng.standard_normal((C, dt.dim)).astype(np.float32).astype(np.float64)
            u = rng.random(C)
            st, info = kern(Draws(z, u), st, dt, h, 6)
            rec.append((_np(st.position), _np(st.logdensity), _np(info.is_accepted),
                        _np(info.energy), _np(info.fixed_point_iters)))
        out[g] = rec
    for a, b in zip(out[1], out[groups]):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


def test_logreg_batched_pdl_bitwise():
    """Programmatic dependent launch only moves each kernel's set-up ahead of
    its predecessor's end: transitions are bit-identical with it on or off
    (a missing wait before a global access would show here)."""
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    kw = dict(N=700, d=25, seed=4)
    dt = device_target("logreg", "mixed", **kw)
    C = 1024
    q0 = start_positions(dt.dim, C, seed=2, scale=0.2).astype(np.float32).astype(np.float64)
    out = {}
    for pdl in (False, True):
        kern = gj.rmhmc.build_kernel(loop="graph", pdl=pdl)
        st = gj.rmhmc.init(q0, dt)
        rng = np.random.Generator(np.random.PCG64(9))
        rec = []
        for h in (0.05, 0.03, 0.05):
            z = rng.standard_normal((C, dt.dim)).astype(np.float32).astype(np.float64)
            u = rng.random(C)
            st, info = kern(Draws(z, u), st, dt, h, 8)
            rec.append((_np(st.position), _np(st.logdensity), _np(st.logdensity_grad),
                        _np(info.energy), _np(info.fixed_point_iters)))
        out[pdl] = rec
    for a, b in zip(out[False], out[True]):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
