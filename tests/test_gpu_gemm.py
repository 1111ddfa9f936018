"""The split-BF16 contraction D = A·Bᵀ (three-term hi/lo product, FP32
accumulation) through the C-ABI test hook, SIMT and tcgen05 kernels, against
a float64 reference of the same split arithmetic and against the exact
product.  Shapes cover the ragged edges the dense-Fisher path meets
(K = d = 25, K = P = 325, N = d, M not a multiple of 128)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SHAPES = [(128, 128, 64), (256, 1000, 25), (200, 325, 1000), (384, 1000, 325), (300, 25, 777),
          (4096, 336, 1000)]


def _pieces(x, planes):
    out = []
    r = x.clone()
    for _ in range(planes):
        b = r.to(torch.bfloat16)
        out.append(b.double())
        r = r - b.float()
    return out


def _split_ref(A, B, planes):
    a = _pieces(A, planes)
    b = _pieces(B, planes)
    ref = torch.zeros(A.shape[0], B.shape[0], dtype=torch.float64, device=A.device)
    for i in range(planes):
        for j in range(planes - i):
            ref += a[i] @ b[j].T
    return ref


def _run(impl, planes, A, B):
    from geomjax_gb300 import _lib as L

    lib = L.lib()
    M, K = A.shape
    N = B.shape[0]
    D = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(lib.gj_gemm_split_bf16(impl, planes, M, N, K, A.data_ptr(), B.data_ptr(), D.data_ptr(), s))
    return D


@pytest.mark.parametrize("planes", [2, 3])
@pytest.mark.parametrize("M,N,K", SHAPES)
def test_gemm_simt(M, N, K, planes):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    D = _run(1, planes, A, B).double()
    exact = A.double() @ B.double().T
    scale = (A.double().abs() @ B.double().abs().T)
    assert torch.max((D - exact).abs() / scale).item() < (1e-4 if planes == 2 else 4e-6)


@pytest.mark.parametrize("planes", [2, 3])
@pytest.mark.parametrize("M,N,K", SHAPES)
def test_gemm_tcgen05(M, N, K, planes):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g)
    B = torch.randn(N, K, device="cuda", generator=g)
    D = _run(2, planes, A, B).double()
    assert torch.isfinite(D).all()
    ref = _split_ref(A, B, planes)
    scale = (A.double().abs() @ B.double().abs().T)
    # same split arithmetic: only FP32 accumulation order differs
    assert torch.max((D - ref).abs() / scale).item() < 2e-6
    exact = A.double() @ B.double().T
    # three planes: FP32-exact operands, the error is the FP32 accumulation
    assert torch.max((D - exact).abs() / scale).item() < (1e-4 if planes == 2 else 4e-6)


def test_fma_peak_plausible():
    """gj_fma_peak: FP32 FMA throughput tens of TFLOP/s, FP64 about 1/64 of
    it on GB300 (nominal 1.25 TFLOP/s)."""
    import ctypes

    from geomjax_gb300 import _lib as L

    v32, v64 = ctypes.c_double(0.0), ctypes.c_double(0.0)
    assert L.lib().gj_fma_peak(L.GJ_MIXED, ctypes.byref(v32), None) == L.GJ_OK
    assert L.lib().gj_fma_peak(L.GJ_FP64, ctypes.byref(v64), None) == L.GJ_OK
    assert 20.0 < v32.value < 200.0, v32.value
    assert 0.2 < v64.value < 5.0, v64.value
    assert v64.value < v32.value / 8
