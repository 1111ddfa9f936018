"""Hand-written adjoint kernels of the target operators behind
torch.autograd.Function, checked by torch.autograd.gradcheck (central finite
differences, float64) on the device."""
import pytest

torch = pytest.importorskip("torch")

from tests.helpers import device_target  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = [
    ("funnel", dict(D=3, metric="diag")),
    ("funnel", dict(D=4, metric="pullback")),
    ("logreg", dict(N=40, d=5, seed=2)),
    ("hier", dict(J=5)),
]


@pytest.mark.parametrize("kind,kw", CASES, ids=lambda x: str(x))
def test_operator_adjoints_match_finite_differences(kind, kw):
    from geomjax_gb300 import autodiff as AD

    tg = device_target(kind, "fp64", **kw)
    g = torch.Generator(device="cuda").manual_seed(3)
    q = (0.3 * torch.randn(3, tg.dim, generator=g, device="cuda", dtype=torch.float64)).requires_grad_()
    opts = dict(eps=1e-6, atol=1e-6, rtol=1e-5)
    assert torch.autograd.gradcheck(lambda x: AD.logdensity(tg, x), (q,), **opts)
    assert torch.autograd.gradcheck(lambda x: AD.grad_logdensity(tg, x), (q,), **opts)
    assert torch.autograd.gradcheck(lambda x: AD.metric(tg, x), (q,), **opts)
