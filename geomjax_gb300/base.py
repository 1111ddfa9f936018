"""State / info / algorithm containers mirroring ``geomjax/base.py`` and the
per-sampler NamedTuples of the reference (``rmhmc/rmhmc.py:30-93``,
``lmcmonge/lmc.py:32-98``, ``lmcmc/lmc.py:30-95``).  Fields are torch
tensors on the device, batched over a leading chain axis."""
from __future__ import annotations

from typing import Any, Callable, NamedTuple


class SamplingAlgorithm(NamedTuple):
    """``base.py:88-113``: a pair (init, step)."""

    init: Callable
    step: Callable


class AdaptationAlgorithm(NamedTuple):
    """``base.py:146-149``."""

    run: Callable


class AdaptationResults(NamedTuple):
    state: Any
    parameters: dict


class Draws(NamedTuple):
    """Explicit randomness for one transition: ``z`` [C, d] standard normals
    (the momentum / velocity draw of ``key_momentum``) and ``u`` [C] uniforms
    (the Metropolis test of ``key_integrator``, accept iff u < p_accept)."""

    z: Any
    u: Any


class RMHMCState(NamedTuple):
    position: Any
    logdensity: Any
    logdensity_grad: Any


class Proposal(NamedTuple):
    """The end of the trajectory after the momentum / velocity flip
    (``RMHMCInfo.proposal.state``, ``rmhmc/rmhmc.py:425-437``): ``velocity``
    is −G⁻¹p for RMHMC and −v for LMC, whether or not it was accepted."""

    position: Any
    velocity: Any


class RMHMCInfo(NamedTuple):
    momentum: Any
    acceptance_rate: Any
    is_accepted: Any
    is_divergent: Any
    energy: Any
    num_integration_steps: int
    fixed_point_iters: Any
    status: Any
    proposal: Any = None


class LMCState(NamedTuple):
    position: Any
    logdensity: Any
    logdensity_grad: Any
    volume_adjustment: Any


class LMCInfo(NamedTuple):
    velocity: Any
    acceptance_rate: Any
    is_accepted: Any
    is_divergent: Any
    energy: Any
    num_integration_steps: int
    status: Any
    proposal: Any = None
