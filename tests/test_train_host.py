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


def test_kornia_constants_by_known_answers():
    """Known answers of the SSIM the reference's kornia computes: on constant
    images a and b every local variance is 0, so
    SSIM = (2ab + C1) C2 / ((a^2 + b^2 + C1) C2 + eps) with C1 = 0.01^2,
    C2 = 0.03^2, eps = 1e-12, whatever the window; the loss term is
    clamp((1 - SSIM) / 2, 0, 1)."""
    a, b = 0.3, 0.7
    img1 = torch.full((9, 10, 3), a, dtype=torch.float64)
    img2 = torch.full((9, 10, 3), b, dtype=torch.float64)
    c1, c2 = 0.01 ** 2, 0.03 ** 2
    want = (2 * a * b + c1) * c2 / ((a * a + b * b + c1) * c2 + 1e-12)
    for win in (3, 4, 11):
        s = L.ssim_map(img1, img2, win)
        assert torch.allclose(s, torch.full_like(s, want), rtol=1e-12, atol=0)
    loss = L.photometric_loss(img1, img2, ssim_mult=1.0, win_size=11)
    assert abs(float(loss) - (1 - want) / 2) < 1e-12


def test_kornia_window_shapes():
    """get_gaussian_kernel1d(w, 1.5): odd windows centred on the middle tap,
    even windows on the half-pixel between the two middle taps (symmetric),
    normalised; the 2D window is the outer product."""
    k11 = L.gaussian_window_1d(11)
    x = torch.arange(11, dtype=torch.float64) - 5
    g = torch.exp(-x * x / 4.5)
    assert torch.allclose(k11, g / g.sum(), rtol=0, atol=1e-15)
    k4 = L.gaussian_window_1d(4)
    x = torch.tensor([-1.5, -0.5, 0.5, 1.5], dtype=torch.float64)
    g = torch.exp(-x * x / 4.5)
    assert torch.allclose(k4, g / g.sum(), rtol=0, atol=1e-15) and torch.allclose(k4, k4.flip(0))
    assert torch.allclose(L.gaussian_window(7), torch.outer(L.gaussian_window_1d(7), L.gaussian_window_1d(7)))


def test_kornia_reflect_padding_same_size():
    """filter2d's "reflect" border mirrors without repeating the edge pixel
    and keeps the image size: an impulse in row 1 reaches output row 0 both
    directly and through the mirrored padding row -1 (= row 1); with edge
    repetition row -1 would be row 0, which is zero."""
    img = torch.zeros(1, 1, 6, 8, dtype=torch.float64)
    img[0, 0, 1, 3] = 1.0
    k1 = L.gaussian_window_1d(3)
    p = torch.nn.functional.pad(img, (1, 1, 1, 1), mode="reflect")
    out = torch.nn.functional.conv2d(p, L.gaussian_window(3)[None, None])
    assert out.shape == img.shape
    assert abs(float(out[0, 0, 0, 3]) - float((k1[0] + k1[2]) * k1[1])) < 1e-15
    # and the restatement's SSIM uses exactly this padding: its mu of the impulse image
    a = img[0, 0][..., None].repeat(1, 1, 3)
    mu = L.ssim_map(a, torch.zeros_like(a), 3)  # mu2 = 0: SSIM = C1 (2 s12 + C2) / ((mu1^2 + C1)(s1 + C2))
    assert mu.shape == (3, 6, 8)
