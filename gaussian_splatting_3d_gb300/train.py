"""The training step around the renderer on native kernels (csrc/train.cu).

``photometric_loss(out, gt)`` is the reference's loss (utils/loss.py:5-24):
``ssim_mult * SSIM_loss + (1 - ssim_mult) * L2`` (or L1), with kornia's SSIM
(Gaussian window, sigma 1.5, reflected borders); two tiled native passes compute
the loss and dL/dout, which the autograd backward hands to the renderer.

``FusedAdam`` is torch.optim.Adam as the reference builds it
(gs/sh_renderer.py:720-729: one group per parameter tensor with its own
learning rate, betas (0.9, 0.99)) with every group updated in one launch.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import torch

from . import _lib
from ._torch import check_tensor, ptr, stream_handle


@dataclass
class LossSettings:
    ssim_mult: float = 0.2      # conf key ssim_loss_mult
    win_size: int = 11          # conf key ssim_loss_win_size
    loss_fn: str = "l2"         # conf key loss_fn: "l1" or "l2" (conf/garden_sh.yaml:35)


def photometric_loss_with_grad(out: torch.Tensor, gt: torch.Tensor, settings: LossSettings | None = None):
    """(loss [] on the device, dL/dout [H,W,3]) for HWC float32 images."""
    st = settings or LossSettings()
    if st.loss_fn not in ("l1", "l2"):
        raise NotImplementedError(st.loss_fn)
    out = out.detach().contiguous()
    gt = gt.detach().to(out.device, torch.float32).contiguous()
    check_tensor(out, "out")
    check_tensor(gt, "gt")
    if out.dim() != 3 or out.shape[-1] != 3 or gt.shape != out.shape:
        raise ValueError("out and gt must both be [H, W, 3]")
    H, W = int(out.shape[0]), int(out.shape[1])
    lib = _lib.load()
    ws_bytes = lib.gsx_photometric_loss_workspace_bytes(H, W)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=out.device)
    nb = int(lib.gsx_photometric_loss_blocks(H, W))
    partials = torch.empty(2 * nb, dtype=torch.float32, device=out.device)
    grad = torch.empty_like(out)
    _lib.call("gsx_photometric_loss", ptr(out), ptr(gt), H, W, int(st.win_size), float(st.ssim_mult),
              1 if st.loss_fn == "l2" else 0, ptr(grad), ptr(partials), ptr(ws), ws_bytes,
              stream_handle(out.device))
    n = 3.0 * H * W
    loss = (partials[:nb].double().sum() * (st.ssim_mult / n)
            + partials[nb:].double().sum() * ((1.0 - st.ssim_mult) / n)).float()
    return loss, grad


class _PhotometricLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, out, gt, settings):
        loss, grad = photometric_loss_with_grad(out, gt, settings)
        ctx.save_for_backward(grad)
        return loss

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        return grad * g, None, None


def photometric_loss(out: torch.Tensor, gt: torch.Tensor, settings: LossSettings | None = None) -> torch.Tensor:
    """The reference's training loss, differentiable with respect to `out`."""
    return _PhotometricLoss.apply(out, gt, settings or LossSettings())


class GsxAdamGroup(ctypes.Structure):
    _fields_ = [("param", ctypes.c_void_p), ("grad", ctypes.c_void_p), ("exp_avg", ctypes.c_void_p),
                ("exp_avg_sq", ctypes.c_void_p), ("n", ctypes.c_int64), ("step_size", ctypes.c_float),
                ("bias_correction2_sqrt", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float),
                ("eps", ctypes.c_float), ("reserved", ctypes.c_int32)]


class FusedAdam(torch.optim.Optimizer):
    """torch.optim.Adam (no weight decay, no amsgrad) with all groups updated
    by one native launch.  Parameters must be float32, contiguous, on one
    CUDA device; a group whose parameters have no gradient is skipped, as
    torch skips them."""

    def __init__(self, params, lr=1e-3, betas=(0.9, 0.99), eps=1e-8):
        super().__init__(params, dict(lr=lr, betas=betas, eps=eps))
        lib = _lib.load()
        if lib.gsx_adam_group_size() != ctypes.sizeof(GsxAdamGroup):
            raise ImportError("gsx_adam_group layout mismatch")

    @torch.no_grad()
    def step(self, closure=None):
        loss = closure() if closure is not None else None
        entries, dev = [], None
        for group in self.param_groups:
            b1, b2 = group["betas"]
            for p in group["params"]:
                if p.grad is None:
                    continue
                check_tensor(p, "param")
                check_tensor(p.grad, "grad")
                st = self.state[p]
                if not st:
                    st["step"] = 0
                    st["exp_avg"] = torch.zeros_like(p)
                    st["exp_avg_sq"] = torch.zeros_like(p)
                st["step"] += 1
                t = st["step"]
                e = GsxAdamGroup()
                e.param, e.grad = ptr(p), ptr(p.grad)
                e.exp_avg, e.exp_avg_sq = ptr(st["exp_avg"]), ptr(st["exp_avg_sq"])
                e.n = p.numel()
                e.step_size = group["lr"] / (1.0 - b1 ** t)
                e.bias_correction2_sqrt = math.sqrt(1.0 - b2 ** t)
                e.beta1, e.beta2, e.eps = b1, b2, group["eps"]
                entries.append(e)
                dev = p.device
        if not entries:
            return loss
        table = (GsxAdamGroup * len(entries))(*entries)
        offs, acc = [], 0
        for e in entries:
            offs.append(acc)
            acc += e.n
        raw = torch.frombuffer(bytearray(bytes(table)), dtype=torch.uint8).pin_memory()
        offsets = torch.tensor(offs, dtype=torch.int64).pin_memory()
        table_dev = raw.to(dev, non_blocking=True)
        offsets_dev = offsets.to(dev, non_blocking=True)
        _lib.call("gsx_adam_step", ptr(table_dev), ptr(offsets_dev), len(entries), acc, stream_handle(dev))
        self._keep = (raw, offsets, table_dev, offsets_dev)  # alive until the copies and the launch have run
        return loss
