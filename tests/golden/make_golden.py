"""Generate the golden per-step fixtures of the float64 oracle.

The reference (JAX) cannot be imported here, so the fixtures come from the
oracle restatement in ``oracle/`` and serve as (1) a regression pin of the
oracle itself (CPU tests) and (2) device-vs-fixture parity without running the
oracle (GPU tests).  Each case stores the inputs (start positions, normals z,
uniforms u, parameters) and, per integration step 1..L, the proposal's
positions, log densities and gradients, plus the final energy and the
accept decisions of one full transition.

Run: ``python tests/golden/make_golden.py`` (writes ``tests/golden/*.npz``).
"""
from __future__ import annotations

import os
import sys

import numpy as np
import zlib

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import lmc as O_lmc  # noqa: E402
from oracle import lmcmonge as O_monge  # noqa: E402
from oracle import rmhmc as O_rm  # noqa: E402
from oracle import targets as OT  # noqa: E402

CASES = {
    # plain FP64 configuration: funnel D=2, diagonal Fisher, h=0.1, 10 steps,
    # 6 fixed-point iterations, 4 chains from ones(2)
    "rmhmc_funnel2_diag": dict(sampler="rmhmc", target=("funnel", dict(D=2, metric="diag")),
                               C=4, h=0.1, L=10, max_iters=6, start="ones", f32=False),
    "rmhmc_funnel2_diag_gl": dict(sampler="rmhmc", integrator="generalized_leapfrog",
                                  target=("funnel", dict(D=2, metric="diag")), C=4, h=0.1, L=10,
                                  max_iters=6, start="ones", f32=False),
    # dense Fisher logistic regression (reduced N, d so the fixture stays small)
    "rmhmc_logreg_n200_d8": dict(sampler="rmhmc", target=("logreg", dict(N=200, d=8, seed=0)),
                                 C=16, h=0.05, L=8, max_iters=100, start="small", f32=True),
    # LMC on a Monge patch, funnel D=100, alpha^2 = 1
    "lmcmonge_funnel100": dict(sampler="lmcmonge", target=("funnel", dict(D=100, metric="diag")),
                               C=8, h=0.02, L=16, alpha2=1.0, start="half", f32=True),
    # dense-metric LMC on the funnel pull-back metric (examples/funnel/main.py)
    "lmc_funnel2_pullback": dict(sampler="lmc", target=("funnel", dict(D=2, metric="pullback")),
                                 C=8, h=0.1, L=8, start="ones", f32=False),
}


def _target(kind, kw):
    if kind == "funnel":
        return OT.Funnel(D=kw["D"], metric=kw["metric"])
    X, y = OT.make_logreg_data(kw["N"], kw["d"], seed=kw["seed"])
    return OT.LogisticRegression(X, y)


def make(name, spec):
    tg = _target(*spec["target"])
    C, d = spec["C"], tg.dim
    rng = np.random.Generator(np.random.PCG64(zlib.crc32(name.encode())))
    if spec["start"] == "ones":
        q0 = np.ones((C, d))
    elif spec["start"] == "half":
        q0 = np.full((C, d), 0.5) + 0.1 * rng.standard_normal((C, d))
    else:
        q0 = 0.2 * rng.standard_normal((C, d))
    z = rng.standard_normal((C, d))
    u = rng.random(C)
    if spec["f32"]:
        q0 = q0.astype(np.float32).astype(np.float64)
        z = z.astype(np.float32).astype(np.float64)
    traj = []
    s = spec["sampler"]
    if s == "rmhmc":
        new, info = O_rm.kernel(tg, O_rm.init(tg, q0), z, u, spec["h"], spec["L"],
                                integrator=spec.get("integrator", "implicit_midpoint"),
                                max_iters=spec.get("max_iters", 100), trajectory=traj)
    elif s == "lmcmonge":
        new, info = O_monge.kernel(tg, O_monge.init(tg, q0), z, u, spec["h"], np.ones(d), spec["L"],
                                   alpha2=spec["alpha2"], trajectory=traj)
    else:
        new, info = O_lmc.kernel(tg, O_lmc.init(tg, q0), z, u, spec["h"], spec["L"], trajectory=traj)
    out = dict(
        q0=q0, z=z, u=u, h=spec["h"], L=spec["L"],
        positions=np.stack([t.position for t in traj]),
        logdensity=np.stack([t.logdensity for t in traj]),
        energy=info.energy, accepted=info.is_accepted, acceptance_rate=info.acceptance_rate,
        new_position=new.position,
    )
    if s == "rmhmc":
        out["momentum0"] = info.momentum
        out["fixed_point_iters"] = info.fixed_point_iters
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


if __name__ == "__main__":
    for n, sp in CASES.items():
        make(n, sp)
        print("wrote", n)
