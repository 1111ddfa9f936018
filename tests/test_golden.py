"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle reproduces its committed fixtures (regression pin).
GPU: the CUDA path reproduces the fixtures without running the oracle —
per-step proposals (forced accept) and one full transition with the stored
uniforms (positions, energy, accept decisions)."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")


def _load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def _cases():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


@pytest.mark.parametrize("name", ["rmhmc_funnel2_diag", "rmhmc_funnel2_diag_gl", "rmhmc_logreg_n200_d8",
                                  "lmcmonge_funnel100", "lmc_funnel2_pullback"])
def test_oracle_reproduces_golden(name, tmp_path, monkeypatch):
    mg = _cases()
    monkeypatch.setattr(mg, "HERE", str(tmp_path))
    mg.make(name, mg.CASES[name])
    new = dict(np.load(os.path.join(tmp_path, name + ".npz")))
    old = _load(name)
    assert set(new) == set(old)
    for k in old:
        np.testing.assert_allclose(new[k], old[k], rtol=1e-12, atol=1e-12, err_msg=k)


def _device(name, spec, precision):
    import geomjax_gb300 as gj
    from geomjax_gb300.data import logreg_data

    kind, kw = spec["target"]
    if kind == "funnel":
        return gj.funnel(D=kw["D"], metric=kw["metric"], precision=precision)
    X, y = logreg_data(kw["N"], kw["d"], seed=kw["seed"])
    return gj.logistic_regression(X, y, precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["rmhmc_funnel2_diag", "rmhmc_funnel2_diag_gl", "rmhmc_logreg_n200_d8",
                                  "lmcmonge_funnel100", "lmc_funnel2_pullback"])
def test_device_matches_golden(name):
    import torch

    import geomjax_gb300 as gj
    from geomjax_gb300.base import Draws

    mg = _cases()
    spec = mg.CASES[name]
    g = _load(name)
    precision = "mixed" if spec["f32"] else "fp64"
    tol = 1e-5 if precision == "mixed" else 1e-10
    dt = _device(name, spec, precision)
    s = spec["sampler"]
    h, L = float(g["h"]), int(g["L"])
    kw = {}
    if s == "rmhmc":
        kern = gj.rmhmc.build_kernel(integrator=spec.get("integrator", "implicit_midpoint"),
                                     max_iters=spec.get("max_iters", 100))
        init = gj.rmhmc.init
    elif s == "lmcmonge":
        kern = gj.lmcmonge.build_kernel()
        init = gj.lmcmonge.init
        kw = dict(alpha2=spec["alpha2"], inverse_mass_matrix=torch.ones(dt.dim, device="cuda"))
    else:
        kern = gj.lmc.build_kernel()
        init = gj.lmc.init
    st0 = init(g["q0"], dt)
    force = -np.ones(len(g["u"]))
    err = lambda a, b: np.max(np.abs(a - b) / (1 + np.abs(b)))  # noqa: E731
    for step in sorted({1, 2, L // 2, L}):
        st, _ = kern(Draws(g["z"], force), st0, dt, h, step, **kw)
        assert err(st.position.double().cpu().numpy(), g["positions"][step - 1]) < tol, step
    st, info = kern(Draws(g["z"], g["u"]), st0, dt, h, L, **kw)
    acc = info.is_accepted.cpu().numpy()
    assert np.array_equal(acc, g["accepted"])
    assert err(st.position.double().cpu().numpy(), g["new_position"]) < tol
    assert err(info.energy.cpu().numpy(), g["energy"]) < tol * 100
