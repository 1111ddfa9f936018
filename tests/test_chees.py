"""ChEES adaptation host logic (CPU): the Halton jitter, the Adam optimiser
and the adaptation update of ``geomjax_gb300.chees`` against the oracle's
restatement of ``adaptation/chees_adaptation_riemanian.py``, and the
oracle's cross-chain statistics against values worked by hand."""
import math

import numpy as np
import pytest

from oracle import chees as OC


def test_halton_sequence_matches_oracle_and_definition():
    from geomjax_gb300.chees import halton_sequence

    bits = math.ceil(math.log2(2000))
    for i in range(0, 3000, 7):
        assert halton_sequence(i, bits) == OC.halton_sequence(i, bits)
    # radical inverse of i + 1: 1 -> 1/2, 2 -> 1/4, 3 -> 3/4, 4 -> 1/8, 6 -> 3/8
    assert [halton_sequence(i) for i in range(6)] == [0.5, 0.25, 0.75, 0.125, 0.625, 0.375]


def test_adam_first_steps():
    from geomjax_gb300.chees import adam

    opt = adam(0.1)
    s = opt.init(1.0)
    # first step: m̂ = g, v̂ = g², update = −lr·g/(|g| + eps)
    u, s = opt.update(3.0, s)
    assert u == pytest.approx(-0.1 * 3.0 / (3.0 + 1e-8), rel=1e-15)
    os_ = OC.adam_init(1.0)
    ou, os_ = OC.adam_update(3.0, os_, 0.1)
    assert u == ou
    rng = np.random.default_rng(0)
    for _ in range(50):
        g = float(rng.standard_normal() * 10)
        u, s = opt.update(g, s)
        ou, os_ = OC.adam_update(g, os_, 0.1)
        assert u == pytest.approx(ou, rel=1e-14, abs=1e-300)
    sched = adam(lambda count: 0.1 / (1 + count))
    s = sched.init(0.0)
    u0, s = sched.update(1.0, s)
    u1, s = sched.update(1.0, s)
    assert u0 == pytest.approx(-0.1, rel=1e-7) and u1 == pytest.approx(-0.05, rel=1e-7)


def test_update_sequence_matches_oracle():
    """50 updates from the same statistics: step size, trajectory length and
    their moving averages agree with the oracle's compute_parameters."""
    from geomjax_gb300.chees import ChEESStatistics, adam, chees_init, chees_update, halton_sequence

    rng = np.random.default_rng(1)
    opt = adam(0.025)
    s = chees_init(0, 0.1, opt)
    o = OC.init(0, 0.1)
    bits = 11
    for i in range(50):
        h = float(rng.uniform(0.2, 1.0))
        g = float(rng.standard_normal() * 5.0)
        jit = halton_sequence(s.random_generator_arg, bits)
        s = chees_update(s, ChEESStatistics(h, g, 0.0), jit, opt, lambda a: a + 1)
        o = OC.compute_parameters(o, h, g, OC.halton_sequence(o.random_generator_arg, bits), 0.025)
        for a, b in [(s.step_size, o.step_size), (s.trajectory_length, o.trajectory_length),
                     (s.log_step_size_moving_average, o.log_step_size_moving_average),
                     (s.log_trajectory_length_moving_average,
                      o.log_trajectory_length_moving_average)]:
            assert a == pytest.approx(b, rel=1e-12, abs=1e-15), i
        assert s.random_generator_arg == o.random_generator_arg == i + 1
        assert s.step == o.step == i + 2


def test_update_keeps_state_on_non_finite_statistics():
    """A NaN harmonic mean (every chain divergent) keeps the dual-averaging
    state and the step size; a NaN gradient keeps log T and the optimiser
    state (chees_adaptation_riemanian.py:149-154, :196-202)."""
    from geomjax_gb300.chees import ChEESStatistics, adam, chees_init, chees_update

    opt = adam(0.025)
    s0 = chees_init(0, 0.1, opt)
    s = chees_update(s0, ChEESStatistics(math.nan, math.nan, 0.0), 0.5, opt, lambda a: a + 1)
    assert s.step_size == 0.1 and s.da_state == s0.da_state
    assert s.optim_state == s0.optim_state
    assert s.trajectory_length == pytest.approx(0.1, rel=1e-15)
    assert s.log_step_size_moving_average == pytest.approx(math.log(0.1), rel=1e-15)


def test_oracle_statistics_by_hand():
    P = np.array([[1.0, 0.0], [0.0, 1.0], [np.nan, 2.0]])
    V = np.array([[1.0, 1.0], [0.5, -1.0], [1.0, 1.0]])
    I = np.array([[0.0, 0.0], [1.0, 1.0], [2.0, 2.0]])
    acc = np.array([0.5, 1.0, 0.2])
    div = np.array([False, False, True])
    h, g, ga = OC.statistics(P, V, I, acc, div, D=V)
    assert h == pytest.approx(1.0 / np.mean([2.0, 1.0]))
    # nanmean: P̄ = (0.5, 1.0), Ī = (1, 1)
    Pc = np.array([[0.5, -1.0], [-0.5, 0.0]])
    Ic = np.array([[-1.0, -1.0], [0.0, 0.0]])
    sq = (Pc ** 2).sum(1) - (Ic ** 2).sum(1)
    gg = sq * (Pc * V[:2]).sum(1)
    assert g == pytest.approx((0.5 * gg[0] + 1.0 * gg[1]) / 1.5)
    assert ga == pytest.approx(g)
    # every chain divergent: NaN harmonic mean and gradient
    h, g, _ = OC.statistics(P, V, I, acc, np.ones(3, dtype=bool))
    assert math.isnan(h) and math.isnan(g)


def test_alpha2_update_sequence_matches_oracle():
    """With update_alpha, α² follows its own Adam step on log α² and moving
    average (chees_adaptation_lmcmonge.py:219-256), as the oracle's."""
    from geomjax_gb300.chees import ChEESStatistics, adam, chees_init, chees_update

    rng = np.random.default_rng(2)
    opt = adam(0.05)
    s = chees_init(0, 0.02, opt, alpha2=0.3)
    o = OC.init(0, 0.02, alpha2=0.3)
    for i in range(40):
        h, g, ga = float(rng.uniform(0.3, 1.0)), float(rng.normal()), float(rng.normal() * 3)
        jit = float(rng.uniform(0.1, 1.0))
        s = chees_update(s, ChEESStatistics(h, g, ga), jit, opt, lambda a: a + 1,
                         update_alpha=True)
        o = OC.compute_parameters(o, h, g, jit, 0.05, grad_alpha_raw=ga)
        assert s.alpha2 == pytest.approx(o.alpha2, rel=1e-12), i
        assert s.step_size == pytest.approx(o.step_size, rel=1e-12)
        assert s.trajectory_length == pytest.approx(o.trajectory_length, rel=1e-12)
    # without update_alpha α² stays where it started
    s = chees_update(chees_init(0, 0.02, opt, alpha2=0.3), ChEESStatistics(0.5, 1.0, 9.0), 0.5,
                     opt, lambda a: a + 1)
    assert s.alpha2 == 0.3


def test_bad_dynamics_rejected():
    import geomjax_gb300 as gj

    with pytest.raises(ValueError):
        gj.chees_adaptation(None, 4, dynamics="nuts")
