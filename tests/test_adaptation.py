"""Host-side adaptation logic (CPU): Stan window schedule, dual averaging and
Welford estimates against direct restatements of the reference formulas."""
import math

import numpy as np
import pytest
import torch

from geomjax_gb300 import adaptation as A


def test_schedule_matches_reference_windows():
    s = A.build_schedule(1000)
    assert len(s) == 1000
    stages = [x[0] for x in s]
    ends = [i for i, x in enumerate(s) if x[1]]
    assert all(x == 0 for x in stages[:75]) and all(x == 0 for x in stages[-50:])
    # windows of 25, 50, 100, 200, 500 (the last one absorbs the rest)
    assert ends == [99, 149, 249, 449, 949]
    assert A.build_schedule(10) == [(0, False)] * 10
    s = A.build_schedule(100)  # resized buffers: 15 fast, 75 slow, 10 fast
    assert sum(x[0] for x in s) == 75 and s[89] == (1, True)


def test_dual_averaging_reaches_target():
    """acceptance(ε) = exp(−ε): the averaged iterate drives the mean
    acceptance to the target 0.8 -> ε* = −log 0.8."""
    s = A.dual_averaging_init(1.0)
    for _ in range(4000):
        eps = math.exp(s.log_step_size)
        s = A.dual_averaging_update(s, 0.8 - math.exp(-eps))
    assert abs(math.exp(s.log_step_size_avg) + math.log(0.8)) < 0.01


def test_dual_averaging_first_step_matches_formula():
    s = A.dual_averaging_init(0.5)
    assert s.mu == pytest.approx(math.log(5.0))
    s1 = A.dual_averaging_update(s, 0.3)
    reg = 1 + 10
    avg = 0.3 / reg
    assert s1.avg_error == pytest.approx(avg)
    assert s1.log_step_size == pytest.approx(math.log(5.0) - (1.0 / 0.05) * avg)
    assert s1.log_step_size_avg == pytest.approx(math.log(0.5))


@pytest.mark.parametrize("diagonal", [True, False])
def test_welford(diagonal):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((37, 4)) @ rng.standard_normal((4, 4))
    s = A.welford_init(4, diagonal)
    s = A.welford_update(s, torch.tensor(x[:20]))
    s = A.welford_update(s, torch.tensor(x[20:]))
    cov, n, mean = A.welford_covariance(s)
    ref = np.cov(x.T, ddof=1)
    assert n == 37
    np.testing.assert_allclose(mean.numpy(), x.mean(0), rtol=1e-12)
    np.testing.assert_allclose(cov.numpy(), np.diag(ref) if diagonal else ref, rtol=1e-10)
    im = A.regularized_inverse_mass(s).numpy()
    exp = (37 / 42) * (np.diag(ref) if diagonal else ref) + 1e-3 * (5 / 42) * (1 if diagonal else np.eye(4))
    np.testing.assert_allclose(im, exp, rtol=1e-10)


@pytest.mark.parametrize("diagonal", [True, False])
def test_welford_batch_equals_one_sample_per_call(diagonal):
    """Folding a [C, d] batch in at once gives the reference's one-sample
    recursion (mass_matrix.py:206-230), restated here row by row."""
    rng = np.random.default_rng(1)
    x = rng.standard_normal((300, 5)) * 3.0 + 10.0
    s = A.welford_init(5, diagonal)
    for blk in (x[:1], x[1:130], x[130:131], x[131:]):
        s = A.welford_update(s, torch.tensor(blk))
    mean = np.zeros(5)
    m2 = np.zeros(5) if diagonal else np.zeros((5, 5))
    for n, v in enumerate(x, start=1):
        delta = v - mean
        mean = mean + delta / n
        upd = v - mean
        m2 = m2 + (delta * upd if diagonal else np.outer(upd, delta))
    assert s.count == 300
    np.testing.assert_allclose(s.mean.numpy(), mean, rtol=1e-13)
    np.testing.assert_allclose(s.m2.numpy(), m2, rtol=1e-11)


def test_gradient_step_size_adaptation_brackets_and_converges(monkeypatch):
    """The safeguarded Newton iteration on a synthetic acceptance curve: a
    smooth decreasing p(h) with a chain that diverges (contributing NaN)
    beyond h = 0.6 reaches the target, and non-finite chains count as
    rejected."""
    import torch

    from geomjax_gb300 import adaptation as A
    from geomjax_gb300 import autodiff as AD

    C = 8

    def fake_jacobian(target, q0, z, h, lam, L, kp, kq):
        p = torch.full((C,), float(np.exp(-(h / 0.3) ** 2)), dtype=torch.float64)
        dp = torch.full((C,), float(-2 * h / 0.09 * np.exp(-(h / 0.3) ** 2)), dtype=torch.float64)
        J = torch.zeros(C, 6, dtype=torch.float64)
        J[:, 0], J[:, 1] = p, dp
        if h > 0.6:
            J[0, :] = float("nan")
        return J

    class FakeTarget:
        device = "cpu"
        prior_var = 100.0

    monkeypatch.setattr(AD, "transition_jacobian", fake_jacobian)
    res = A.gradient_step_size_adaptation(FakeTarget(), np.zeros((C, 3)), 5, initial_step_size=0.01,
                                          target_acceptance_rate=0.5, tol=1e-8)
    h_star = 0.3 * np.sqrt(np.log(2.0))
    assert abs(res.step_size - h_star) < 1e-6 and abs(res.mean_acceptance - 0.5) < 1e-8
    # from far above the root: the NaN chain counts as rejected, the bracket still closes
    res = A.gradient_step_size_adaptation(FakeTarget(), np.zeros((C, 3)), 5, initial_step_size=2.0,
                                          target_acceptance_rate=0.5, tol=1e-8)
    assert abs(res.step_size - h_star) < 1e-6
    assert any(np.isfinite(pa) and pa < 1.0 / C + 1e-12 for _, pa, _ in res.history)
