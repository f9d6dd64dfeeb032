"""FP64 restatement of the reference's training loss (utils/loss.py:5-24).

TEST INFRASTRUCTURE ONLY (the checker of csrc/train.cu's loss kernels).

The reference calls kornia.losses.ssim_loss, which is not installed here;
this follows kornia's published definition (kornia.metrics.ssim with a
normalised Gaussian window of sigma 1.5, per-channel 2D filtering with
reflected borders and "same" output size, C1 = (0.01 max_val)^2,
C2 = (0.03 max_val)^2, max_val 1, SSIM = num / (den + eps), eps 1e-12; loss =
mean(clamp((1 - SSIM) / 2, 0, 1))).  Its version is unpinned in the
reference (requirements.txt), so the SSIM term's parity is unpinned; torch
autograd of this function is the gradient reference.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F


def gaussian_window(win_size: int, sigma: float = 1.5, dtype=torch.float64, device="cpu"):
    x = torch.arange(win_size, dtype=dtype, device=device) - (win_size // 2)
    g = torch.exp(-x * x / (2.0 * sigma * sigma))
    g = g / g.sum()
    return g[:, None] * g[None, :]


def ssim_map(img1, img2, win_size: int = 11):
    """img1, img2: [H, W, 3] -> [3, H, W] SSIM map."""
    a = img1.permute(2, 0, 1)[None]
    b = img2.permute(2, 0, 1)[None]
    k = gaussian_window(win_size, dtype=a.dtype, device=a.device)[None, None].repeat(3, 1, 1, 1)
    r = win_size // 2

    def filt(x):
        return F.conv2d(F.pad(x, (r, r, r, r), mode="reflect"), k, groups=3)

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
