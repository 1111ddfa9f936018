"""Batches of uneven logistic-regression posteriors (``gj_batch_*``): every
posterior's chains follow the oracle step by step, and the batch (one CUDA
graph holding every posterior as a branch, one CUDA graph of grouped
launches over all posteriors, or one graph per posterior on a stream pool)
is bit-identical to running each posterior on its own."""
import numpy as np
import pytest

from tests.helpers import normals, rel_err, start_positions

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

# the largest d (the path's maximum, 128) first: a later, smaller context
# must not lower the process-wide shared-memory limit the larger one's
# launches need
SIZES = [(220, 128), (200, 8), (350, 21), (260, 40)]
C = 64


def _data():
    from geomjax_gb300.data import logreg_data

    return [logreg_data(N, d, seed=10 + i) for i, (N, d) in enumerate(SIZES)]


def _starts():
    return [start_positions(d, C, seed=20 + i, scale=0.2).astype(np.float32).astype(np.float64)
            for i, (_, d) in enumerate(SIZES)]


def _draws(seed):
    zs, us = [], []
    for i, (_, d) in enumerate(SIZES):
        z, u = normals(C, d, seed + i, np.float32)
        zs.append(z)
        us.append(u)
    return zs, us


def _np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("integrator", ["implicit_midpoint", "generalized_leapfrog"])
def test_batch_matches_oracle_per_posterior(integrator):
    from geomjax_gb300.base import Draws
    from geomjax_gb300.batch import PosteriorBatch
    from oracle import rmhmc as O_rm
    from oracle import targets as OT

    data = _data()
    pb = PosteriorBatch(data, C, num_streams=3, integrator=integrator)
    q0 = _starts()
    zs, _ = _draws(7)
    us = [-np.ones(C) for _ in SIZES]  # accept every proposal: compare trajectories
    h = 0.05
    for L in (1, 4):
        st = pb.init(q0)
        st, info = pb.step(Draws(np.concatenate([z.ravel() for z in zs]), np.concatenate(us)), st,
                           h, L)
        for b, (X, y) in enumerate(data):
            ot = OT.LogisticRegression(X, y, prior_var=100.0)
            traj = []
            _, oi = O_rm.kernel(ot, O_rm.init(ot, q0[b]), zs[b], us[b], h, L, trajectory=traj,
                                integrator=integrator)
            e = rel_err(_np(pb.positions(st, b)), traj[-1].position)
            assert e < 1e-5, (b, L, e)
            eb = _np(info.energy)[b * C:(b + 1) * C]
            assert rel_err(eb, oi.energy) < 1e-4, (b, L)


@pytest.mark.parametrize("one_graph,grouped", [(True, False), (True, True), (False, False)])
def test_batch_bitwise_equals_single_posterior_runs(one_graph, grouped):
    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws
    from geomjax_gb300.batch import PosteriorBatch

    data = _data()
    pb = PosteriorBatch(data, C, num_streams=4, one_graph=one_graph, grouped=grouped)
    q0 = _starts()
    zs, us = _draws(11)
    st = pb.init(q0)
    st, info = pb.step(Draws(np.concatenate([z.ravel() for z in zs]), np.concatenate(us)), st,
                       0.05, 6)
    kern = gj.rmhmc.build_kernel(loop="graph")
    for b, (X, y) in enumerate(data):
        t = gj.logistic_regression(X, y, precision="mixed")
        s1, i1 = kern(Draws(zs[b], us[b]), gj.rmhmc.init(q0[b], t), t, 0.05, 6)
        np.testing.assert_array_equal(_np(pb.positions(st, b)), _np(s1.position))
        np.testing.assert_array_equal(_np(st.logdensity)[b * C:(b + 1) * C], _np(s1.logdensity))
        np.testing.assert_array_equal(_np(info.is_accepted)[b * C:(b + 1) * C],
                                      _np(i1.is_accepted))
        np.testing.assert_array_equal(_np(info.fixed_point_iters)[b * C:(b + 1) * C],
                                      _np(i1.fixed_point_iters))


@pytest.mark.parametrize("integrator", ["implicit_midpoint", "generalized_leapfrog"])
def test_batch_one_graph_reused_across_calls(integrator):
    """The one-graph batch, as branches and as grouped launches (one bucket
    and three buckets of posteriors), over three transitions (the graph captured at the first is reused, the step size
    changes between calls, the state arrays move) equals the stream-pool
    batch bit for bit, info included."""
    import torch
    from geomjax_gb300.batch import PosteriorBatch

    data = _data()
    outs = []
    for one, grouped, buckets in ((True, False, 0), (True, True, 0), (True, True, 3),
                                  (False, False, 0)):
        pb = PosteriorBatch(data, C, num_streams=3, one_graph=one, grouped=grouped,
                            buckets=buckets, integrator=integrator)
        st = pb.init(_starts())
        info = pb.new_info()
        g = torch.Generator(device="cuda").manual_seed(5)
        n = int(pb.offsets[-1])
        rec = []
        for h in (0.05, 0.04, 0.06):
            z = torch.randn(n, generator=g, device="cuda")
            u = torch.rand(len(SIZES) * C, generator=g, device="cuda", dtype=torch.float64)
            st = type(st)(*(t.clone() for t in st))  # new addresses every call
            pb.step_inplace(st, z, u, info, h, 5)
            rec.append([_np(st.position), _np(st.logdensity), _np(st.logdensity_grad)] +
                       [_np(info[k]) for k in ("acceptance_rate", "is_accepted", "energy",
                                               "fp_iters", "status", "momentum")])
        outs.append(rec)
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            for x, y in zip(a, b):
                np.testing.assert_array_equal(x, y)
