"""Training-step kernels against their references.

* photometric loss: value within 1e-5 relative and dL/dout within 1e-4 *
  max |reference| of torch autograd through the FP64 restatement of the
  reference's loss (oracle/loss_ref.py), for L1 and L2, windows 11 and 7,
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
@pytest.mark.parametrize("hw", [(48, 64), (135, 240)])
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
    shapes = [(1000, 3), (1000, 4), (1000, 3), (1000, 3, 16), (1000,)]
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
