"""CPU float64 oracle for the geomjax sampler hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
package; only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline``
/ ``--impl reference`` legs of ``bench.py`` may use it, and only as the checker
or as the timed CPU baseline.

The reference (williwilliams3/geomjax) is pure Python on JAX.  JAX is not
installed here and cannot be, so the reference cannot be executed.  This
package restates the reference algorithms line by line in NumPy float64,
batched over a leading chain axis (the reference batches with ``jax.vmap``).
Every function cites the reference file:line it follows.

Randomness: the reference draws ``normal(key_momentum)`` and
``bernoulli(key_integrator, p)``.  Here the caller passes host-drawn standard
normals ``z`` and uniforms ``u`` instead, and ``bernoulli(key, p)`` becomes
``u < p`` (that is how ``jax.random.bernoulli`` is defined).

Pinning: the reference's only runnable pins are the structural G = I
equivalences of ``tests/test_samplers.py:21-57`` (RMHMC with G = I equals
HMC velocity Verlet equals dense LMC with G = I, rtol 1e-4).  They are
checked in ``tests/test_oracle.py``.  The golden value at
``tests/test_samplers.py:19`` needs JAX threefry bits and the absent
``postjax`` package, so beyond those structural pins the oracle's parity with
the reference is **unpinned** (see the header of each module for the
invariants that are checked instead: finite-difference derivatives,
reversibility, energy-error order).
"""

from . import targets, proposal, rmhmc, lmcmonge, lmc, hmc, diagnostics  # noqa: F401
