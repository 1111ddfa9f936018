"""The C-ABI library loads and exports every symbol the header declares; host
argument checks reject bad inputs without touching a GPU."""
import ctypes
import os
import re

import pytest

from geomjax_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_symbols():
    text = open(os.path.join(ROOT, "include", "geomjax_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int32_t|int64_t|const char\*)\s+(gj_\w+)\s*\(", text, re.M)))


def test_library_exports_every_header_symbol():
    lib = L.load()
    syms = _header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
        assert s in L.SIGNATURES, f"{s} has no ctypes signature"


def test_version_and_error_strings():
    lib = L.load()
    assert lib.gj_version() >= 100
    assert isinstance(lib.gj_last_error(), bytes)


def test_struct_layouts_match_c(tmp_path):
    """ctypes layouts equal the C compiler's (offsetof / sizeof of the header)."""
    import shutil
    import subprocess

    ours = (ctypes.sizeof(L.GjTarget), L.GjStepParams.tol.offset, L.GjStepParams.inverse_mass.offset,
            ctypes.sizeof(L.GjStepParams), ctypes.sizeof(L.GjChainState), ctypes.sizeof(L.GjInfo))
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        assert ours == (56, 24, 48, 64, 40, 72)
        return
    src = tmp_path / "off.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "geomjax_gb300.h"\n'
        'int main(){printf("%zu %zu %zu %zu %zu %zu", sizeof(gj_target), offsetof(gj_step_params,tol),'
        ' offsetof(gj_step_params,inverse_mass), sizeof(gj_step_params), sizeof(gj_chain_state),'
        ' sizeof(gj_info));}\n')
    exe = tmp_path / "off"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = tuple(int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                               check=True).stdout.split())
    assert got == ours


def test_argument_checks_without_gpu():
    lib = L.load()
    h = ctypes.c_void_p()
    bad = L.GjTarget(99, 1, 2, 0, None, None, None, 3.0, 0.0)
    assert lib.gj_create(ctypes.byref(bad), 0, 0, 4, ctypes.byref(h)) == L.GJ_EINVAL
    assert b"family" in lib.gj_last_error()
    t = L.GjTarget(L.GJ_FUNNEL, L.GJ_METRIC_DIAG_FISHER, 1, 0, None, None, None, 3.0, 0.0)
    assert lib.gj_create(ctypes.byref(t), 0, 0, 4, ctypes.byref(h)) == L.GJ_EINVAL
    t = L.GjTarget(L.GJ_LOGREG, L.GJ_METRIC_DENSE_FISHER, 5, 10, None, None, None, 100.0, 0.0)
    assert lib.gj_create(ctypes.byref(t), 0, 1, 4, ctypes.byref(h)) == L.GJ_EINVAL
    t = L.GjTarget(L.GJ_FUNNEL, L.GJ_METRIC_DIAG_FISHER, 3, 0, None, None, None, 3.0, 0.0)
    assert lib.gj_create(ctypes.byref(t), 7, 0, 4, ctypes.byref(h)) == L.GJ_EINVAL
    assert lib.gj_create(ctypes.byref(t), 0, 0, 0, ctypes.byref(h)) == L.GJ_EINVAL
    # a valid context is pure host state until the first step
    assert lib.gj_create(ctypes.byref(t), 0, 0, 4, ctypes.byref(h)) == L.GJ_OK
    st = L.GjChainState(None, None, None, None, 4)
    p = L.GjStepParams(0.1, 10, 0, 100, 1e-6, 1000.0, 0.0, None, 0, 0)
    assert lib.gj_rmhmc_step(h, ctypes.byref(p), ctypes.byref(st), None, None, None, None) == L.GJ_EINVAL
    assert lib.gj_lmc_step(h, ctypes.byref(p), ctypes.byref(st), None, None, None, None) == L.GJ_EINVAL
    p.num_integration_steps = -1
    assert lib.gj_set_option(h, 999, 0) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_LOGREG_PATH, 9) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_CHOL_CHAINS_PER_WARP, 3) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_CHOL_CHAINS_PER_WARP, 16) == L.GJ_EINVAL
    for v in (0, 1, 2, 4, 8):
        assert lib.gj_set_option(h, L.GJ_OPT_CHOL_CHAINS_PER_WARP, v) == L.GJ_OK
    assert lib.gj_set_option(h, L.GJ_OPT_CHAIN_GROUPS, 9) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_THREADS_PER_BLOCK, 256) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_THREADS_PER_BLOCK, 64) == L.GJ_OK
    assert lib.gj_set_option(h, L.GJ_OPT_PDL, 2) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_PDL, 0) == L.GJ_OK
    assert lib.gj_set_option(h, L.GJ_OPT_GEMM_KSPLIT, 5) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_GEMM_KSPLIT, -1) == L.GJ_EINVAL
    for v in range(5):
        assert lib.gj_set_option(h, L.GJ_OPT_GEMM_KSPLIT, v) == L.GJ_OK
    assert lib.gj_set_option(h, L.GJ_OPT_CHAIN_GROUPS, 2) == L.GJ_OK
    assert lib.gj_set_option(h, L.GJ_OPT_FUSE_R2X, 2) == L.GJ_EINVAL
    assert lib.gj_set_option(h, L.GJ_OPT_FUSE_R2X, -1) == L.GJ_EINVAL
    for v in (0, 1):
        assert lib.gj_set_option(h, L.GJ_OPT_FUSE_R2X, v) == L.GJ_OK
    for v in (-1, 2):
        assert lib.gj_set_option(h, L.GJ_OPT_REFINE_ITERATES, v) == L.GJ_EINVAL
    for v in (0, 1):
        assert lib.gj_set_option(h, L.GJ_OPT_REFINE_ITERATES, v) == L.GJ_OK
    # gj_stats: at most 11 counters (out[8..10]: refined solves, their time,
    # their FP64 fallbacks); a context without the batched path reports one
    # launch per step and nothing else
    stats = (ctypes.c_int64 * 16)(*([-1] * 16))
    assert lib.gj_stats(h, stats, 16) == 11
    assert list(stats[:11]) == [0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0] and stats[11] == -1
    assert lib.gj_stats(h, stats, 4) == 4
    assert lib.gj_stats(None, stats, 4) == L.GJ_EINVAL
    assert lib.gj_set_gemm_tiling(96, 1) == L.GJ_EINVAL
    # batch creation checks its arguments before touching the GPU
    bh = ctypes.c_void_p()
    assert lib.gj_batch_create(None, 1, 64, 4, ctypes.byref(bh)) == L.GJ_EINVAL
    tl = (L.GjTarget * 2)(L.GjTarget(L.GJ_LOGREG, L.GJ_METRIC_DENSE_FISHER, 5, 10, 1, 1, None,
                                     100.0, 0.0),
                          L.GjTarget(L.GJ_FUNNEL, L.GJ_METRIC_DIAG_FISHER, 3, 0, None, None, None,
                                     3.0, 0.0))
    tp = ctypes.cast(tl, ctypes.c_void_p)
    assert lib.gj_batch_create(tp, 0, 64, 4, ctypes.byref(bh)) == L.GJ_EINVAL
    assert lib.gj_batch_create(tp, 1, 0, 4, ctypes.byref(bh)) == L.GJ_EINVAL
    assert lib.gj_batch_create(tp, 1, 64, 0, ctypes.byref(bh)) == L.GJ_EINVAL
    assert lib.gj_batch_create(tp, 2, 64, 4, ctypes.byref(bh)) == L.GJ_EINVAL  # a funnel
    tl[0].dim = 200
    assert lib.gj_batch_create(tp, 1, 64, 4, ctypes.byref(bh)) == L.GJ_ENOTSUP
    assert lib.gj_batch_destroy(None) == L.GJ_OK
    assert lib.gj_set_gemm_tiling(128, 2) == L.GJ_EINVAL
    assert lib.gj_set_gemm_tiling(0, -1) == L.GJ_OK  # back to the automatic policy
    # the differentiated transition checks its arguments on the host
    assert lib.gj_logreg_gl_transition_jvp(None, 1, None, None, 0.1, 0.5, 1, 2, 2, 1, None,
                                           None) == L.GJ_EINVAL
    tl = L.GjTarget(L.GJ_LOGREG, L.GJ_METRIC_DENSE_FISHER, 80, 10, 1, 1, None, 100.0, 0.0)
    assert lib.gj_logreg_gl_transition_jvp(ctypes.byref(tl), 1, 1, 1, 0.1, 0.5, 1, 2, 2, 1, 1,
                                           None) == L.GJ_ENOTSUP
    tl.dim, tl.n_data = 64, 5000  # the per-chain shared memory would exceed 227 KB
    assert lib.gj_logreg_gl_transition_jvp(ctypes.byref(tl), 1, 1, 1, 0.1, 0.5, 1, 2, 2, 1, 1,
                                           None) == L.GJ_ENOTSUP
    tl.n_data = 10
    tl.dim = 5
    assert lib.gj_logreg_gl_transition_jvp(ctypes.byref(tl), 1, 1, 1, 0.1, -1.0, 1, 2, 2, 1, 1,
                                           None) == L.GJ_EINVAL
    assert lib.gj_logreg_gl_transition_jvp(ctypes.byref(tl), 1, 1, 1, 0.1, 0.5, 1, 0, 2, 1, 1,
                                           None) == L.GJ_EINVAL
    # NUTS: host checks on a context (no GPU touched before the launch)
    np_ = L.GjNutsParams(0.1, 17, 0, 0, 100, 1e-6, 1000.0, 0.0, None, 0, 0)
    st4 = L.GjChainState(1, 1, 1, None, 4)
    assert lib.gj_nuts_step(None, ctypes.byref(np_), ctypes.byref(st4), 1, 1, 10**6, None,
                            None) == L.GJ_EINVAL
    assert lib.gj_nuts_step(h, ctypes.byref(np_), ctypes.byref(st4), 1, 1, 10**6, None,
                            None) == L.GJ_EINVAL  # 17 doublings
    np_.max_num_doublings = 4
    np_.criterion = 3
    assert lib.gj_nuts_step(h, ctypes.byref(np_), ctypes.byref(st4), 1, 1, 100, None,
                            None) == L.GJ_EINVAL
    np_.criterion = 0
    assert lib.gj_nuts_step(h, ctypes.byref(np_), ctypes.byref(st4), 1, 1, 2 * 4 + 15 - 1, None,
                            None) == L.GJ_EINVAL  # one uniform short
    assert lib.gj_nuts_step(h, ctypes.byref(np_), ctypes.byref(st4), None, 1, 100, None,
                            None) == L.GJ_EINVAL
    assert lib.gj_fma_peak(5, ctypes.byref(ctypes.c_double()), None) == L.GJ_EINVAL
    # the α² derivative of the LMC-Monge proposal: host checks
    pp = L.GjStepParams(0.02, 8, 0, 0, 0.0, 1000.0, 1.0, None, 0, 0)
    assert lib.gj_lmcmonge_alpha2_jvp(None, 0, 4, ctypes.byref(pp), 1, 1, None, 1,
                                      None) == L.GJ_EINVAL
    tf = L.GjTarget(L.GJ_FUNNEL, L.GJ_METRIC_DIAG_FISHER, 3, 0, None, None, None, 3.0, 0.0)
    assert lib.gj_lmcmonge_alpha2_jvp(ctypes.byref(tf), 0, 4, ctypes.byref(pp), None, 1, None, 1,
                                      None) == L.GJ_EINVAL
    tg = L.GjTarget(L.GJ_LOGREG, L.GJ_METRIC_DENSE_FISHER, 5, 10, 1, 1, None, 100.0, 0.0)
    assert lib.gj_lmcmonge_alpha2_jvp(ctypes.byref(tg), 0, 4, ctypes.byref(pp), 1, 1, None, 1,
                                      None) == L.GJ_ENOTSUP
    # ChEES statistics: workspace size and host checks
    assert lib.gj_chees_workspace_size(4096, 25) == 8 * (2 * 25 + 5 * 4096)
    assert lib.gj_chees_workspace_size(0, 25) == -1
    assert lib.gj_chees_statistics(7, 4, 2, 1, 1, 1, None, 1, None, 1, 1, None) == L.GJ_EINVAL
    assert lib.gj_chees_statistics(L.GJ_FP64, 0, 2, 1, 1, 1, None, 1, None, 1, 1,
                                   None) == L.GJ_EINVAL
    assert lib.gj_chees_statistics(L.GJ_FP64, 4, 2, None, 1, 1, None, 1, None, 1, 1,
                                   None) == L.GJ_EINVAL
    assert lib.gj_chees_statistics(L.GJ_FP64, 4, 2, 1, 1, 1, None, 1, None, None, 1,
                                   None) == L.GJ_EINVAL
    assert lib.gj_gemm_split_bf16(3, 2, 1, 1, 1, None, None, None, None) == L.GJ_EINVAL
    assert lib.gj_gemm_split_bf16(1, 4, 1, 1, 1, None, None, None, None) == L.GJ_EINVAL
    assert lib.gj_destroy(h) == L.GJ_OK


def test_no_cpu_fallback():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import geomjax_gb300 as gj

    with pytest.raises(L.GeomjaxError):
        gj.funnel(D=2, precision="fp64", device="cpu").logdensity_and_grad([[0.0, 0.0]])
