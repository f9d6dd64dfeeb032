"""The FP64 loss restatement on the CPU: SSIM of an image with itself is 1,
the loss is 0 there, the window is a normalised Gaussian, and the function is
differentiable as torch autograd sees it (gradcheck on a small image)."""
import pytest

torch = pytest.importorskip("torch")

from oracle import loss_ref as L  # noqa: E402


def test_window_and_identity():
    k = L.gaussian_window(11)
    assert abs(float(k.sum()) - 1.0) < 1e-12 and torch.allclose(k, k.T)
    g = torch.Generator().manual_seed(0)
    img = torch.rand(20, 17, 3, generator=g, dtype=torch.float64)
    s = L.ssim_map(img, img)
    assert torch.allclose(s, torch.ones_like(s), atol=1e-9)
    assert float(L.photometric_loss(img, img)) < 1e-9


def test_gradcheck_small():
    g = torch.Generator().manual_seed(1)
    out = torch.rand(13, 12, 3, generator=g, dtype=torch.float64, requires_grad=True)
    gt = torch.rand(13, 12, 3, generator=g, dtype=torch.float64)
    for fn in ("l1", "l2"):
        assert torch.autograd.gradcheck(lambda o: L.photometric_loss(o, gt, 0.2, 7, fn), (out,), eps=1e-6,
                                        atol=1e-6)
