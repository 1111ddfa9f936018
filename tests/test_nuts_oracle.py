"""The NUTS oracle (CPU): the checkpoint index arithmetic of the iterative
U-turn criterion against the reference's worked examples, and the
structural pin that one expansion of NUTS is one RMHMC step with a
Metropolis accept."""
import numpy as np
import pytest

from oracle import nuts as ON
from oracle import rmhmc as O_rm
from tests.helpers import oracle_target, start_positions


def test_checkpoint_indices_match_reference_examples():
    # termination.py:80-90: "6 -> 2, 7 -> 2, 13 -> 2" set bits of n >> 1 and
    # "6 -> 0, 7 -> 3, 13 -> 1" trailing ones
    for n, hi, ones in [(6, 2, 0), (7, 2, 3), (13, 2, 1), (0, 0, 0), (1, 0, 1)]:
        lo, h = ON.leaf_idx_to_ckpt_idxs(n)
        assert h == hi and lo == hi - ones + 1


def test_num_uniforms():
    assert ON.num_uniforms(10) == 2 * 10 + 1023
    assert ON.num_uniforms(1) == 3


@pytest.mark.parametrize("direction", [1, -1])
@pytest.mark.parametrize("kind,kw", [("funnel", dict(D=2, metric="diag")),
                                     ("logreg", dict(N=30, d=3))], ids=str)
def test_one_expansion_is_one_rmhmc_step(kind, kw, direction):
    """max_num_doublings = 1: the trajectory is one integrator step in the
    drawn direction and the biased merge accepts it with probability
    min(e^{H0 − H1}, 1), the RMHMC kernel's accept with L = 1 and step
    direction · h."""
    ot = oracle_target(kind, **kw)
    C = 6
    q0 = start_positions(ot.dim, C, seed=2, scale=0.4)
    rng = np.random.default_rng(5)
    z = rng.standard_normal((C, ot.dim))
    ua = rng.random(C)
    u = np.stack([np.full(C, 0.25 if direction > 0 else 0.75), ua, np.zeros(C)], axis=1)
    st = O_rm.init(ot, q0)
    new_n, infos = ON.kernel(ot, st, z, u, 0.1, 1)
    new_r, info_r = O_rm.kernel(ot, st, z, ua, direction * 0.1, 1)
    np.testing.assert_allclose(new_n.position, new_r.position, rtol=0, atol=1e-14)
    np.testing.assert_allclose([i.acceptance_rate for i in infos], info_r.acceptance_rate,
                               rtol=1e-13)
    assert all(i.num_integration_steps == 1 and i.num_trajectory_expansions == 1 for i in infos)


@pytest.mark.parametrize("dynamics", ["lmc", "lmcmonge"])
def test_one_expansion_is_one_lmc_step(dynamics):
    """The same pin for the LMC samplers: one expansion is one lan step with
    the static Metropolis accept (lmcmc/lmc.py:411-476, lmcmonge/lmc.py:
    472-536), the volume adjustment included."""
    from oracle import lmc as O_lmc
    from oracle import lmcmonge as O_mo

    kind, kw = ("funnel", dict(D=3, metric="pullback")) if dynamics == "lmc" else \
        ("funnel", dict(D=5, metric="diag"))
    ot = oracle_target(kind, **kw)
    C = 5
    q0 = start_positions(ot.dim, C, seed=4, scale=0.4)
    rng = np.random.default_rng(7)
    z = rng.standard_normal((C, ot.dim))
    ua = rng.random(C)
    u = np.stack([np.full(C, 0.25), ua, np.zeros(C)], axis=1)
    im = np.linspace(0.9, 1.1, ot.dim)
    if dynamics == "lmc":
        st = O_lmc.init(ot, q0)
        st.volume_adjustment = rng.standard_normal(C) * 0.1
        new_n, infos = ON.kernel(ot, st, z, u, 0.05, 1, dynamics="lmc")
        new_r, info_r = O_lmc.kernel(ot, st, z, ua, 0.05, 1)
    else:
        st = O_mo.init(ot, q0)
        new_n, infos = ON.kernel(ot, st, z, u, 0.05, 1, dynamics="lmcmonge", alpha2=0.5,
                                 inverse_mass_matrix=im)
        new_r, info_r = O_mo.kernel(ot, st, z, ua, 0.05, im, 1, alpha2=0.5)
    np.testing.assert_allclose(new_n.position, new_r.position, rtol=0, atol=1e-13)
    np.testing.assert_allclose(new_n.volume_adjustment, new_r.volume_adjustment, atol=1e-13)
    np.testing.assert_allclose(new_n.logdensity_grad, new_r.logdensity_grad, atol=1e-12)
    np.testing.assert_allclose([i.acceptance_rate for i in infos], info_r.acceptance_rate,
                               rtol=1e-12)
