"""Training-step kernels against their references.

* photometric loss: value within 1e-5 relative and dL/dout within 1e-4 *
  max |reference| of torch autograd through the FP64 restatement of the
  reference's loss with the kornia 0.6 series' SSIM (oracle/loss_ref.py;
  utils/loss.py:15-20 calls kornia.losses.ssim_loss), for L1 and L2, windows
  11 (the reference's configuration) and 7,
  images with identical regions (the clamp and the L1 kink);
* FusedAdam: three steps with per-group learning rates equal torch.optim.Adam
  (the reference's optimizer, betas (0.9, 0.99)) within 1e-6 relative.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import train  # noqa: E402
from oracle import loss_ref as L  # noqa: E402

pytestmark = pytest.mark.gpu


def dev():
    return torch.device("cuda:0")


@pytest.mark.parametrize("loss_fn", ["l1", "l2"])
@pytest.mark.parametrize("win", [11, 7])
@pytest.mark.parametrize("hw", [(48, 64), (135, 240), (271, 481)])
def test_photometric_loss_matches_fp64(loss_fn, win, hw):
    g = torch.Generator().manual_seed(1000 * win + hw[0] + (loss_fn == "l2"))
    H, W = hw
    out = torch.rand(H, W, 3, generator=g)
    gt = torch.rand(H, W, 3, generator=g)
    gt[: H // 3] = out[: H // 3]  # identical rows: SSIM 1 there, L1 at its kink
    st = train.LossSettings(ssim_mult=0.2, win_size=win, loss_fn=loss_fn)
    loss, grad = train.photometric_loss_with_grad(out.to(dev()), gt.to(dev()), st)
    o64 = out.double().requires_grad_(True)
    ref = L.photometric_loss(o64, gt.double(), 0.2, win, loss_fn)
    ref.backward()
    assert abs(float(loss) - float(ref.detach())) <= 1e-5 * abs(float(ref.detach()))
    r = o64.grad.numpy()
    err = np.abs(grad.cpu().double().numpy() - r).max() / np.abs(r).max()
    assert err <= 1e-4, err


@pytest.mark.parametrize("hw,win", [((1, 4000), 1), ((2, 3000), 3), ((6, 1920), 11)])
def test_photometric_loss_thin_images(hw, win):
    """Fewer partial-sum slots than 32x32 tiles: a CTA walks several tiles."""
    g = torch.Generator().manual_seed(hw[1] + win)
    out = torch.rand(*hw, 3, generator=g)
    gt = torch.rand(*hw, 3, generator=g)
    st = train.LossSettings(ssim_mult=0.2, win_size=win, loss_fn="l2")
    loss, grad = train.photometric_loss_with_grad(out.to(dev()), gt.to(dev()), st)
    o64 = out.double().requires_grad_(True)
    ref = L.photometric_loss(o64, gt.double(), 0.2, win, "l2")
    ref.backward()
    assert abs(float(loss) - float(ref.detach())) <= 1e-5 * abs(float(ref.detach()))
    r = o64.grad.numpy()
    assert np.abs(grad.cpu().double().numpy() - r).max() / np.abs(r).max() <= 1e-4


def test_photometric_loss_autograd_feeds_renderer_gradient():
    g = torch.Generator().manual_seed(3)
    out = torch.rand(40, 50, 3, generator=g).to(dev()).requires_grad_(True)
    gt = torch.rand(40, 50, 3, generator=g).to(dev())
    loss = train.photometric_loss(out, gt)
    (2.0 * loss).backward()
    _, grad = train.photometric_loss_with_grad(out.detach(), gt)
    torch.testing.assert_close(out.grad, 2.0 * grad)


def test_fused_adam_matches_torch_adam():
    g = torch.Generator().manual_seed(4)
    # sizes off the 4-element vectors and the 1024-element blocks
    shapes = [(1000, 3), (1001, 4), (333, 3), (1000, 3, 16), (7,)]
    lrs = [1e-3, 1e-2, 1e-2, 1e-2, 1e-2]
    a = [torch.randn(s, generator=g).to(dev()) for s in shapes]
    b = [t.clone() for t in a]
    pa = [torch.nn.Parameter(t) for t in a]
    pb = [torch.nn.Parameter(t) for t in b]
    opt_a = train.FusedAdam([{"params": [p], "lr": lr} for p, lr in zip(pa, lrs)], betas=(0.9, 0.99))
    opt_b = torch.optim.Adam([{"params": [p], "lr": lr} for p, lr in zip(pb, lrs)], betas=(0.9, 0.99))
    for step in range(3):
        grads = [torch.randn(s, generator=g).to(dev()) * (10.0 ** -step) for s in shapes]
        for p, q, gr in zip(pa, pb, grads):
            p.grad = gr.clone()
            q.grad = gr.clone()
        opt_a.step()
        opt_b.step()
        for p, q in zip(pa, pb):
            torch.testing.assert_close(p.data, q.data, rtol=1e-6, atol=1e-7)


def test_fused_adam_many_groups():
    """More groups than one warp scans at a time (the kernel's group search)."""
    g = torch.Generator().manual_seed(5)
    sizes = [int(s) for s in torch.randint(1, 3000, (70,), generator=g)]
    a = [torch.randn(n, generator=g).to(dev()) for n in sizes]
    pa = [torch.nn.Parameter(t) for t in a]
    pb = [torch.nn.Parameter(t.clone()) for t in a]
    lrs = [1e-3 * (1 + i % 7) for i in range(len(sizes))]
    opt_a = train.FusedAdam([{"params": [p], "lr": lr} for p, lr in zip(pa, lrs)], betas=(0.9, 0.99))
    opt_b = torch.optim.Adam([{"params": [p], "lr": lr} for p, lr in zip(pb, lrs)], betas=(0.9, 0.99))
    for _ in range(2):
        for p, q in zip(pa, pb):
            gr = torch.randn(p.shape, generator=g).to(dev())
            p.grad = gr.clone()
            q.grad = gr.clone()
        opt_a.step()
        opt_b.step()
    for p, q in zip(pa, pb):
        torch.testing.assert_close(p.data, q.data, rtol=1e-6, atol=1e-7)
