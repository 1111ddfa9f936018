"""The generalized leapfrog's position-iterate solves u = G(q_k)⁻¹p½ by
mixed-precision iterative refinement (an FP32 factorisation, corrections from
FP64 residuals p − G·u; GJ_OPT_REFINE_ITERATES, the default) against the same
solves by the FP64 factorisation (GJ_OPT_REFINE_ITERATES = 0), on the
batched mixed path (rmhmc/integrators.py's generalized leapfrog,
rmhmc/metrics.py's dense Fisher metric):

* per-step positions of every chain agree to 2e-7 (relative, 1 added to the
  denominator: a few float32 roundings), fixed-point iteration counts agree,
  and both match the float64 oracle to 1e-5: logistic regression N = 1000, d = 25 (the
  benchmark's data) and N = 2000, d = 64 (the largest d the refinement takes);
* the same with a rank-deficient design (a duplicated column) and prior
  variance 1e5, where G's condition number is about 1e7: the FP32
  factorisation cannot reach an FP64 solve's accuracy there, so the chains
  fall back to the FP64 factorisation (gj_stats out[10] counts them);
* the refined solves are the ones launched (gj_stats out[8]), and none with
  the option off; on the well-conditioned metric none falls back.

The refinement stops when the predicted error of x is below 2⁻⁴⁴‖x‖, under
an FP64 solve's own error, so the two solves differ in their last bits only.
The positions still differ by float32 roundings: each iterate is rounded to
float32 for the next evaluation's contractions, and where two FP64 values a
few ulps apart round to neighbouring float32 values, the evaluations that
follow carry that difference (4e-8 after 5 steps at d = 64 when measured).
Without the refinement (an FP32 solve alone) they would differ by about
κ(G)·d·2⁻²⁴ relative in u.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import rmhmc as O_rm  # noqa: E402
from oracle import targets as OT  # noqa: E402
from tests.helpers import laplace_draws, rel_err  # noqa: E402

pytestmark = pytest.mark.gpu

GL = "generalized_leapfrog"


def _np(t):
    return t.detach().double().cpu().numpy()


def _f32(a):
    return np.asarray(a).astype(np.float32).astype(np.float64)


def _kernels(**kw):
    import geomjax_gb300 as gj

    return (gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=GL, refine_iterates=True, **kw),
            gj.rmhmc.build_kernel(logreg_path="tcgen05", integrator=GL, refine_iterates=False, **kw))


@pytest.mark.parametrize("N,d,C", [(1000, 25, 1024), (2000, 64, 256)])
def test_refined_iterates_match_fp64(N, d, C):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws
    from geomjax_gb300.data import logreg_data

    X, y = logreg_data(N, d, seed=0)
    ot = OT.LogisticRegression(X, y)
    dt = gj.logistic_regression(X, y, precision="mixed")
    S = np.arange(0, C, C // 16)
    q0 = _f32(laplace_draws(ot, C, seed=31))
    z = _f32(np.random.default_rng(32).standard_normal((C, d)))
    u = -np.ones(C)
    h, L = 0.05, 10
    traj = []
    O_rm.kernel(ot, O_rm.init(ot, q0[S]), z[S], u[S], h, L, trajectory=traj, integrator=GL)
    kr, kf = _kernels()
    st0 = gj.rmhmc.init(q0, dt)
    for step in (1, 5, 10):
        sr, ir = kr(Draws(z, u), st0, dt, h, step)
        sf, if_ = kf(Draws(z, u), st0, dt, h, step)
        pr, pf = _np(sr.position), _np(sf.position)
        assert rel_err(pr, pf) < 2e-7, (step, rel_err(pr, pf))
        assert rel_err(pr[S], traj[step - 1].position) < 1e-5
        it_r, it_f = _np(ir.fixed_point_iters), _np(if_.fixed_point_iters)
        assert np.mean(it_r == it_f) >= 0.999, np.mean(it_r == it_f)


def test_refinement_falls_back_on_ill_conditioned_metric():
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws
    from geomjax_gb300.data import logreg_data

    N, d, C = 400, 8, 256
    X, y = logreg_data(N, d, seed=3)
    X[:, 1] = X[:, 0]  # XᵀΛX singular along e0 − e1: there λ(G) = 1/prior_var
    pv = 1e5
    dt = gj.logistic_regression(X, y, prior_var=pv, precision="mixed")
    rng = np.random.default_rng(33)
    q0 = _f32(0.1 * rng.standard_normal((C, d)))
    z = _f32(rng.standard_normal((C, d)))
    u = -np.ones(C)
    kr, kf = _kernels(loop="host")
    ctx = kr.context(dt, C)
    assert ctx.lib.gj_profile(ctx.h, 1) == 0  # counts the fallbacks
    st0 = gj.rmhmc.init(q0, dt)
    sr, _ = kr(Draws(z, u), st0, dt, 0.01, 3)
    buf = (ctypes.c_int64 * 11)()
    assert ctx.lib.gj_stats(ctx.h, buf, 11) == 11
    assert ctx.lib.gj_profile(ctx.h, 0) == 0
    sf, _ = kf(Draws(z, u), st0, dt, 0.01, 3)
    pr, pf = _np(sr.position), _np(sf.position)
    assert np.all(np.isfinite(pr))
    assert rel_err(pr, pf) < 2e-7, rel_err(pr, pf)
    assert buf[10] > 0, list(buf)  # chains fell back to the FP64 factorisation


def test_refined_solves_are_launched():
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws
    from geomjax_gb300.data import logreg_data

    X, y = logreg_data(300, 9, seed=0)
    dt = gj.logistic_regression(X, y, precision="mixed")
    C = 128
    rng = np.random.default_rng(34)
    q0 = _f32(0.1 * rng.standard_normal((C, 9)))
    z = _f32(rng.standard_normal((C, 9)))
    counts = []
    for kern in _kernels(loop="host"):
        ctx = kern.context(dt, C)
        assert ctx.lib.gj_profile(ctx.h, 1) == 0
        kern(Draws(z, -np.ones(C)), gj.rmhmc.init(q0, dt), dt, 0.05, 4)
        buf = (ctypes.c_int64 * 11)()
        assert ctx.lib.gj_stats(ctx.h, buf, 11) == 11
        assert ctx.lib.gj_profile(ctx.h, 0) == 0
        counts.append((buf[5], buf[8], buf[10]))
    (chol_r, ref_r, fb_r), (chol_f, ref_f, fb_f) = counts
    assert ref_r > 0 and ref_f == 0, counts
    assert 0 < chol_r < chol_f, counts  # the full evaluations still factor in FP64
    assert fb_r == 0 and fb_f == 0, counts
