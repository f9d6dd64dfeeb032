"""Tensor checks and raw pointers for the C ABI (torch is plumbing only)."""
from __future__ import annotations

import torch


def check_tensor(t: torch.Tensor, name: str, dtype: torch.dtype | None = torch.float32,
                 cuda: bool = True) -> None:
    """Raise RuntimeError like the reference's CHECK_* macros (gs/src/include/common.h:29-54)."""
    if not isinstance(t, torch.Tensor):
        raise RuntimeError(f"{name} must be a tensor")
    if cuda and not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise RuntimeError(f"{name} must be a contiguous tensor")
    if dtype is not None and t.dtype != dtype:
        kind = {torch.float32: "a floating", torch.int32: "an int", torch.bool: "an bool"}.get(dtype, str(dtype))
        raise RuntimeError(f"{name} must be {kind} tensor")


def ptr(t: torch.Tensor | None) -> int | None:
    if t is None:
        return None
    return t.data_ptr() if t.numel() > 0 else None


def stream_handle(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream
