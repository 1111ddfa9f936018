"""The no-allocation contraction entry point (gj_gemm_split_bf16_noalloc).

Callers such as an XLA custom call, whose framework already reserved the
device memory for its own pool, cannot call cudaMalloc; this entry point
keeps its scratch in a static device array instead.  The test checks it
against the allocating entry point gj_gemm_split_bf16 on two calls in a row
(different shapes, so the second call runs over the first call's leftovers
in the shared array), through the C ABI, and against the float64 product of
the same inputs; and that sizes beyond the array's capacity are rejected.
It lives in its own file, which pytest collects last."""
import ctypes

import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _call(fn, impl, planes, A, B):
    from geomjax_gb300 import _lib as L

    M, K = A.shape
    N = B.shape[0]
    D = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(fn(impl, planes, M, N, K, A.data_ptr(), B.data_ptr(), D.data_ptr(), s))
    return D


@pytest.mark.parametrize("impl", [2, 1])
def test_noalloc_matches_allocating_entry_point(impl):
    from geomjax_gb300 import _lib as L

    if impl == 2 and torch.cuda.get_device_capability()[0] != 10:
        pytest.skip("the tcgen05 contraction needs a Blackwell (sm_10x) device")

    lib = L.lib()
    g = torch.Generator(device="cuda").manual_seed(7)
    cases = [(3, 384, 1000, 325), (2, 200, 130, 777)]  # (planes, M, N, K)
    for planes, M, N, K in cases:
        A = torch.randn(M, K, device="cuda", generator=g)
        B = torch.randn(N, K, device="cuda", generator=g)
        ref = _call(lib.gj_gemm_split_bf16, impl, planes, A, B).double()
        got = _call(lib.gj_gemm_split_bf16_noalloc, impl, planes, A, B).double()
        exact = A.double() @ B.double().T
        scale = A.double().abs() @ B.double().abs().T
        assert torch.isfinite(got).all()
        # same split arithmetic and the same kernels: only the scratch differs
        assert torch.max((got - ref).abs() / scale).item() < 1e-6
        # and both are the float64 product to the split planes' resolution
        # (2 planes: 16 mantissa bits per operand, 3 planes: 24)
        tol = 1e-4 if planes == 2 else 4e-6
        assert torch.max((got - exact).abs() / scale).item() < tol


def test_noalloc_rejects_oversized_problems():
    from geomjax_gb300 import _lib as L

    lib = L.lib()
    A = torch.zeros(4096, 1024, device="cuda")
    B = torch.zeros(4096, 1024, device="cuda")
    D = torch.zeros(4096, 4096, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.gj_gemm_split_bf16_noalloc(2, 2, 4096, 4096, 1024, A.data_ptr(), B.data_ptr(),
                                        D.data_ptr(), s)
    assert rc == L.GJ_EINVAL
    assert b"4194304" in lib.gj_last_error()
