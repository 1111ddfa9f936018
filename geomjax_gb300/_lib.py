"""ctypes binding of the C ABI declared in ``include/geomjax_gb300.h``.

The shared library is built in-tree by ``geomjax_gb300.build`` into
``geomjax_gb300/_build/libgeomjax_gb300.so``.  There is no CPU fallback: if
the library or a CUDA device is missing, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_double, c_int32, c_int64, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgeomjax_gb300.so")

# enums (include/geomjax_gb300.h)
GJ_OK, GJ_EINVAL, GJ_ENOTSUP, GJ_ECUDA, GJ_ENOMEM = 0, 1, 2, 3, 4
GJ_FUNNEL, GJ_LOGREG, GJ_HIERGAUSS = 1, 2, 3
GJ_METRIC_DIAG_FISHER, GJ_METRIC_DENSE_FISHER, GJ_METRIC_PULLBACK, GJ_METRIC_IDENTITY = 1, 2, 3, 4
GJ_FP64, GJ_MIXED = 0, 1
GJ_IMPLICIT_MIDPOINT, GJ_GENERALIZED_LEAPFROG = 0, 1
GJ_SAMPLER_RMHMC, GJ_SAMPLER_LMC, GJ_SAMPLER_LMCMONGE = 0, 1, 2
GJ_CHAIN_FP_NOT_CONVERGED, GJ_CHAIN_NONFINITE, GJ_CHAIN_NOT_SPD = 0x1, 0x2, 0x4
GJ_OPT_LOGREG_PATH, GJ_OPT_THREADS_PER_BLOCK, GJ_OPT_LOOP, GJ_OPT_CHOL_FP64 = 1, 2, 3, 4
GJ_OPT_CHOL_CHAINS_PER_WARP, GJ_OPT_CHAIN_GROUPS, GJ_OPT_PDL = 5, 6, 7
GJ_OPT_GEMM_KSPLIT = 8
GJ_OPT_BATCH_GRAPH = 9
GJ_OPT_MONGE_WARP = 10
GJ_OPT_FUSE_R2X = 11
GJ_OPT_BATCH_BUCKETS = 12
GJ_OPT_REFINE_ITERATES = 13


class GjTarget(ctypes.Structure):
    _fields_ = [
        ("family", c_int32),
        ("metric", c_int32),
        ("dim", c_int32),
        ("n_data", c_int32),
        ("X", c_void_p),
        ("y", c_void_p),
        ("s", c_void_p),
        ("p0", c_double),
        ("p1", c_double),
    ]


class GjChainState(ctypes.Structure):
    _fields_ = [
        ("position", c_void_p),
        ("logdensity_grad", c_void_p),
        ("logdensity", c_void_p),
        ("volume_adjustment", c_void_p),
        ("num_chains", c_int32),
    ]


# GjInfo's fields in order, as keys of the samplers' info dicts
INFO_FIELDS = ("acceptance_rate", "is_accepted", "is_divergent", "energy", "fp_iters", "status",
               "momentum", "proposal_position", "proposal_velocity")


class GjInfo(ctypes.Structure):
    _fields_ = [
        ("acceptance_rate", c_void_p),
        ("is_accepted", c_void_p),
        ("is_divergent", c_void_p),
        ("energy", c_void_p),
        ("fp_iters", c_void_p),
        ("status", c_void_p),
        ("momentum", c_void_p),
        ("proposal_position", c_void_p),
        ("proposal_velocity", c_void_p),
    ]


class GjStepParams(ctypes.Structure):
    _fields_ = [
        ("step_size", c_double),
        ("num_integration_steps", c_int32),
        ("integrator", c_int32),
        ("max_iters", c_int32),
        ("tol", c_double),
        ("divergence_threshold", c_double),
        ("alpha2", c_double),
        ("inverse_mass", c_void_p),
        ("alpha2_fix", c_int32),
        ("reserved", c_int32),
    ]


class GjNutsParams(ctypes.Structure):
    _fields_ = [
        ("step_size", c_double),
        ("max_num_doublings", c_int32),
        ("integrator", c_int32),
        ("criterion", c_int32),
        ("max_iters", c_int32),
        ("tol", c_double),
        ("divergence_threshold", c_double),
        ("alpha2", c_double),
        ("inverse_mass", c_void_p),
        ("alpha2_fix", c_int32),
        ("reserved", c_int32),
    ]


# GjNutsInfo's fields in order, as keys of the NUTS info dicts
NUTS_INFO_FIELDS = ("acceptance_rate", "is_divergent", "is_turning", "energy",
                    "num_trajectory_expansions", "num_integration_steps", "fp_iters", "status",
                    "momentum", "leftmost_position", "rightmost_position")


class GjNutsInfo(ctypes.Structure):
    _fields_ = [(k, c_void_p) for k in NUTS_INFO_FIELDS]


# every symbol the header declares, with its ctypes signature
SIGNATURES = {
    "gj_version": (c_int32, []),
    "gj_last_error": (ctypes.c_char_p, []),
    "gj_create": (c_int32, [POINTER(GjTarget), c_int32, c_int32, c_int32, POINTER(c_void_p)]),
    "gj_destroy": (c_int32, [c_void_p]),
    "gj_set_option": (c_int32, [c_void_p, c_int32, c_int64]),
    "gj_init": (c_int32, [c_void_p, POINTER(GjChainState), c_void_p]),
    "gj_rmhmc_step": (c_int32, [c_void_p, POINTER(GjStepParams), POINTER(GjChainState), c_void_p,
                                c_void_p, POINTER(GjInfo), c_void_p]),
    "gj_lmcmonge_step": (c_int32, [c_void_p, POINTER(GjStepParams), POINTER(GjChainState),
                                   c_void_p, c_void_p, POINTER(GjInfo), c_void_p]),
    "gj_lmc_step": (c_int32, [c_void_p, POINTER(GjStepParams), POINTER(GjChainState), c_void_p,
                              c_void_p, POINTER(GjInfo), c_void_p]),
    "gj_nuts_step": (c_int32, [c_void_p, POINTER(GjNutsParams), POINTER(GjChainState),
                                     c_void_p, c_void_p, c_int32, POINTER(GjNutsInfo), c_void_p]),
    "gj_stats": (c_int32, [c_void_p, POINTER(c_int64), c_int32]),
    "gj_profile": (c_int32, [c_void_p, c_int32]),
    "gj_gemm_split_bf16": (c_int32, [c_int32, c_int32, c_int32, c_int32, c_int32, c_void_p,
                                     c_void_p, c_void_p, c_void_p]),
    "gj_gemm_split_bf16_noalloc": (c_int32, [c_int32, c_int32, c_int32, c_int32, c_int32,
                                             c_void_p, c_void_p, c_void_p, c_void_p]),
    "gj_logdensity_grad": (c_int32, [POINTER(GjTarget), c_int32, c_int32, c_void_p, c_void_p,
                                     c_void_p, c_void_p]),
    "gj_hvp": (c_int32, [POINTER(GjTarget), c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                         c_void_p]),
    "gj_metric": (c_int32, [POINTER(GjTarget), c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    "gj_set_gemm_tiling": (c_int32, [c_int32, c_int32]),
    "gj_batch_create": (c_int32, [c_void_p, c_int32, c_int32, c_int32, POINTER(c_void_p)]),
    "gj_batch_destroy": (c_int32, [c_void_p]),
    "gj_batch_set_option": (c_int32, [c_void_p, c_int32, c_int64]),
    "gj_batch_rmhmc_step": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p]),
    "gj_logreg_gl_transition_jvp": (c_int32, [POINTER(GjTarget), c_int32, c_void_p, c_void_p,
                                              c_double, c_double, c_int32, c_int32, c_int32,
                                              c_int32, c_void_p, c_void_p]),
    "gj_lmcmonge_alpha2_jvp": (c_int32, [POINTER(GjTarget), c_int32, c_int32,
                                         POINTER(GjStepParams), c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p]),
    "gj_fma_peak": (c_int32, [c_int32, POINTER(c_double), c_void_p]),
    "gj_set_gemm_accumulators": (c_int32, [c_int32]),
    "gj_chees_workspace_size": (c_int64, [c_int32, c_int32]),
    "gj_chees_statistics": (c_int32, [c_int32, c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p]),
    "gj_metric_vjp": (c_int32, [POINTER(GjTarget), c_int32, c_int32, c_void_p, c_void_p, c_void_p,
                                c_void_p]),
}


class GeomjaxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"geomjax_gb300 error {code}: {msg}")
        self.code = code


_LIB = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the shared library (no device needed) and bind every symbol."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise GeomjaxError(GJ_ENOTSUP, f"CUDA library not built: {path} (run geomjax_gb300.build)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def lib() -> ctypes.CDLL:
    """The library, for compute calls: requires a CUDA device."""
    import torch

    if not torch.cuda.is_available():
        raise GeomjaxError(GJ_ENOTSUP, "no CUDA device: geomjax_gb300 has no CPU fallback")
    return load()


def check(rc: int):
    if rc != GJ_OK:
        raise GeomjaxError(rc, _LIB.gj_last_error().decode(errors="replace"))


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()
