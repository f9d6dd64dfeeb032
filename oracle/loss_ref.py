"""FP64 restatement of the reference's training loss (utils/loss.py:5-24).

TEST INFRASTRUCTURE ONLY (the checker of csrc/train.cu's loss kernels).

The reference calls kornia.losses.ssim_loss(out, gt, ssim_loss_win_size,
reduction="mean") (utils/loss.py:2, 15-20; window 11 in
conf/garden_sh.yaml:38).  kornia is not installed here and its version is
not pinned in requirements.txt, but the reference also imports
kornia.geometry.conversions.QuaternionCoeffOrder (utils/transforms.py:5),
which only the kornia 0.6 series still exports, so this restates the SSIM
loss of that series as its source defines it:

* kornia.losses.ssim_loss(img1, img2, window_size, max_val=1.0, eps=1e-12,
  reduction="mean", padding="same") = mean(clamp((1 - ssim_map) / 2, 0, 1));
* kornia.metrics.ssim: window = get_gaussian_kernel2d((w, w), (1.5, 1.5)),
  the outer product of the 1D kernel x = arange(w) - w // 2 (+ 0.5 when w is
  even), g = exp(-x^2 / (2 sigma^2)) / sum; each of img1, img2, img1^2,
  img2^2, img1*img2 filtered per channel by kornia.filters.filter2d with
  border_type "reflect" (torch's reflect padding, (w - 1) // 2 before and the
  rest after, "same" output size); C1 = (0.01 max_val)^2,
  C2 = (0.03 max_val)^2; sigma1^2 = E[img1^2] - mu1^2 (likewise sigma2^2,
  sigma12); ssim_map = (2 mu1 mu2 + C1)(2 sigma12 + C2) /
  ((mu1^2 + mu2^2 + C1)(sigma1^2 + sigma2^2 + C2) + eps).

No kornia output exists here to compare against, so the constants and the
structure are pinned by known-answer tests (tests/test_train_host.py) instead;
torch autograd of this function is the gradient reference.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F


def gaussian_window_1d(win_size: int, sigma: float = 1.5, dtype=torch.float64, device="cpu"):
    x = torch.arange(win_size, dtype=dtype, device=device) - (win_size // 2)
    if win_size % 2 == 0:
        x = x + 0.5
    g = torch.exp(-x * x / (2.0 * sigma * sigma))
    return g / g.sum()


def gaussian_window(win_size: int, sigma: float = 1.5, dtype=torch.float64, device="cpu"):
    g = gaussian_window_1d(win_size, sigma, dtype, device)
    return g[:, None] * g[None, :]


def ssim_map(img1, img2, win_size: int = 11):
    """img1, img2: [H, W, 3] -> [3, H, W] SSIM map."""
    a = img1.permute(2, 0, 1)[None]
    b = img2.permute(2, 0, 1)[None]
    k = gaussian_window(win_size, dtype=a.dtype, device=a.device)[None, None].repeat(3, 1, 1, 1)
    front = (win_size - 1) // 2
    rear = win_size - 1 - front

    def filt(x):
        return F.conv2d(F.pad(x, (front, rear, front, rear), mode="reflect"), k, groups=3)

    mu1, mu2 = filt(a), filt(b)
    s1 = filt(a * a) - mu1 * mu1
    s2 = filt(b * b) - mu2 * mu2
    s12 = filt(a * b) - mu1 * mu2
    c1, c2 = 1e-4, 9e-4
    num = (2 * mu1 * mu2 + c1) * (2 * s12 + c2)
    den = (mu1 * mu1 + mu2 * mu2 + c1) * (s1 + s2 + c2)
    return (num / (den + 1e-12))[0]


def photometric_loss(out, gt, ssim_mult: float = 0.2, win_size: int = 11, loss_fn: str = "l2"):
    ssim_l = torch.clamp((1.0 - ssim_map(out, gt, win_size)) / 2, 0.0, 1.0).mean()
    base = F.mse_loss(out, gt) if loss_fn == "l2" else F.l1_loss(out, gt)
    return ssim_mult * ssim_l + (1.0 - ssim_mult) * base
