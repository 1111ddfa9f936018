"""The launch-choice autotuner: it times every candidate on a copy of the
state, leaves the fastest set, and the kernel then runs with it."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from tests.helpers import device_target, start_positions  # noqa: E402

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().double().cpu().numpy()


def test_autotune_batched_logreg_keeps_state_and_results():
    import geomjax_gb300 as gj
    from geomjax_gb300 import _lib as L
    from geomjax_gb300.base import Draws

    dt = device_target("logreg", "mixed", N=300, d=6, seed=1)
    C = 256
    q0 = start_positions(6, C, seed=2, scale=0.2)
    kern = gj.rmhmc.build_kernel()
    st = gj.rmhmc.init(q0, dt)
    before = [t.clone() for t in st]
    res = gj.autotune(kern, dt, st, 0.05, 4, transitions=2, tilings=((0, -1), (0, 1)),
                      chol_chains_per_warp=(0, 2), gemm_ksplit=(0, 2))
    for a, b in zip(before, st):
        assert torch.equal(a, b)  # the state is not advanced
    # four first-stage candidates, then K split 2 with the best of them
    assert len(res.table) == 5 and res.best in [c for c, _ in res.table]
    assert res.table[4][0]["gemm_ksplit"] == 2
    assert {k: v for k, v in res.table[4][0].items() if k != "gemm_ksplit"} == \
        {k: v for k, v in min(res.table[:4], key=lambda x: x[1])[0].items() if k != "gemm_ksplit"}
    assert res.ms_per_transition == min(ms for _, ms in res.table) > 0
    # the chosen settings are in force and give the same transition as the
    # defaults up to the order of floating-point sums
    z = np.random.default_rng(3).standard_normal((C, 6)).astype(np.float32)
    u = np.random.default_rng(4).random(C)
    s1, i1 = kern(Draws(z, u), st, dt, 0.05, 4)
    L.check(L.lib().gj_set_gemm_tiling(0, -1))
    k0 = gj.rmhmc.build_kernel()
    s0, i0 = k0(Draws(z, u), st, dt, 0.05, 4)
    assert np.max(np.abs(_np(s1.position) - _np(s0.position))) < 1e-5
    assert (np.asarray(_np(i1.is_accepted)) == np.asarray(_np(i0.is_accepted))).mean() > 0.99


def test_autotune_per_chain_threads():
    import geomjax_gb300 as gj

    dt = device_target("funnel", "fp64", D=2, metric="diag")
    kern = gj.rmhmc.build_kernel(max_iters=6)
    st = gj.rmhmc.init(np.ones((512, 2)), dt)
    res = gj.autotune(kern, dt, st, 0.1, 4, transitions=2)
    assert {c["threads_per_block"] for c, _ in res.table} == {32, 64, 128}


def test_autotune_batch():
    import geomjax_gb300 as gj
    from geomjax_gb300 import _lib as L
    from geomjax_gb300.batch import PosteriorBatch
    from geomjax_gb300.data import logreg_data

    data = [logreg_data(200, 8, seed=1), logreg_data(350, 21, seed=2)]
    pb = PosteriorBatch(data, 64, num_streams=2)
    st = pb.init([0.01 * np.ones((64, 8)), 0.01 * np.ones((64, 21))])
    res = gj.autotune_batch(pb, st, 0.05, 3, transitions=1, tilings=((0, -1), (64, -1)),
                            chol_chains_per_warp=(0, 2), gemm_ksplit=(0, 1))
    assert len(res.table) == 5
    new, info = pb.step(1, st, 0.05, 3)
    assert np.isfinite(_np(new.position)).all()
    L.check(L.lib().gj_set_gemm_tiling(0, -1))
