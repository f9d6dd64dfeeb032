"""Drop-in replacement for the reference's compiled module ``_gs``.

The reference imports its CUDA extension as ``import _gs as _backend``
(gs/renderer.py:20-23, gs/sh_renderer.py:24-27).  Registering this module
under that name, e.g. ``sys.modules["_gs"] = gaussian_splatting_3d_gb300._gs``,
routes the reference's Python code to the sm_103a kernels.  The four
hot-path functions keep the reference's positional signatures
(gs/src/render.h:3-5, 65-68, 86-101), its in-place output convention and its
RuntimeError on bad tensors (gs/src/include/common.h:29-54).

Differences, all deliberate:
  * every call is enqueued on torch's current CUDA stream (the reference uses
    the legacy default stream for culling and binning);
  * an unsupported SH order C raises instead of silently doing nothing
    (gs/src/render.cu:506-543 has a switch without default);
  * equal (tile, depth) keys are ordered by Gaussian index, where the
    reference's order depends on atomic scheduling (aabb_culling.h:32);
  * scratch memory comes from torch's caching allocator, not per-call
    cudaMalloc/cudaFree (aabb_culling.h:202-259).
"""
from __future__ import annotations

import torch

from . import _lib
from ._torch import check_tensor, ptr, stream_handle


def culling_gaussian_bsphere(mean, qvec, svec, normal, pts, mask, thresh):
    """mask[i] = bounding sphere of Gaussian i intersects the frustum
    (gs/src/render.cu:15-43)."""
    for t, name in ((mean, "mean"), (qvec, "qvec"), (svec, "svec"), (normal, "normal"), (pts, "pts")):
        check_tensor(t, name)
    check_tensor(mask, "mask", torch.bool)
    n = mean.size(0)
    _lib.call("gsx_culling_gaussian_bsphere", n, ptr(mean), ptr(qvec), ptr(svec), ptr(normal),
              ptr(pts), ptr(mask), float(thresh), stream_handle(mean.device))


def tile_culling_aabb_start_end(aabb_topleft, aabb_bottomright, gaussian_ids, start, end, depth,
                                n_tiles_h, n_tiles_w):
    """Sorted (tile, depth) Gaussian lists and per-tile [start, end)
    (gs/src/render.cu:380-397).  Synchronises once, as the reference does."""
    for t, name in ((aabb_topleft, "aabb_topleft"), (aabb_bottomright, "aabb_bottomright"),
                    (gaussian_ids, "gaussian_ids"), (start, "start"), (end, "end")):
        check_tensor(t, name, torch.int32)
    check_tensor(depth, "depth")
    n = aabb_topleft.size(0)
    n_keys = gaussian_ids.size(0)
    n_tiles = int(n_tiles_h) * int(n_tiles_w)
    if start.numel() < n_tiles or end.numel() < n_tiles:
        raise RuntimeError("start and end must hold n_tiles_h * n_tiles_w entries")
    ws_bytes = _lib.load().gsx_binning_workspace_bytes(n, n_keys, n_tiles)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=depth.device)
    _lib.call("gsx_tile_culling_aabb_start_end", n, n_keys, ptr(aabb_topleft), ptr(aabb_bottomright),
              ptr(depth), int(n_tiles_h), int(n_tiles_w), ptr(gaussian_ids), ptr(start), ptr(end),
              ptr(ws), ws_bytes, stream_handle(depth.device))


def _check_raster(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out, topleft, c2w):
    for t, name in ((mean, "mean"), (cov, "cov"), (alpha, "alpha"), (sh_coeffs, "sh_coeffs"),
                    (out, "out"), (topleft, "topleft"), (c2w, "c2w")):
        check_tensor(t, name)
    for t, name in ((start, "start"), (end, "end"), (gaussian_ids, "gaussian_ids")):
        check_tensor(t, name, torch.int32)


def tile_based_vol_rendering_sh(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out, topleft,
                                c2w, tile_size, n_tiles_h, n_tiles_w, pixel_size_x, pixel_size_y, H, W,
                                C, thresh):
    """Forward SH raster into the pre-zeroed ``out`` (gs/src/render.cu:483-544)."""
    _check_raster(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out, topleft, c2w)
    _lib.call("gsx_tile_based_vol_rendering_sh", mean.size(0), gaussian_ids.size(0), ptr(mean),
              ptr(cov), ptr(sh_coeffs), ptr(alpha), ptr(start), ptr(end), ptr(gaussian_ids), ptr(out),
              ptr(topleft), ptr(c2w), int(tile_size), int(n_tiles_h), int(n_tiles_w),
              float(pixel_size_x), float(pixel_size_y), int(H), int(W), int(C), float(thresh),
              stream_handle(mean.device))


def tile_based_vol_rendering_backward_sh(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out,
                                         grad_mean, grad_cov, grad_sh_coeffs, grad_alpha, grad_out,
                                         topleft, c2w, tile_size, n_tiles_h, n_tiles_w, pixel_size_x,
                                         pixel_size_y, H, W, C, thresh):
    """Backward SH raster accumulating into the pre-zeroed grad_* tensors
    (gs/src/render.cu:546-624)."""
    _check_raster(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out, topleft, c2w)
    for t, name in ((grad_mean, "grad_mean"), (grad_cov, "grad_cov"), (grad_sh_coeffs, "grad_sh_coeffs"),
                    (grad_alpha, "grad_alpha"), (grad_out, "grad_out")):
        check_tensor(t, name)
    _lib.call("gsx_tile_based_vol_rendering_backward_sh", mean.size(0), gaussian_ids.size(0), ptr(mean),
              ptr(cov), ptr(sh_coeffs), ptr(alpha), ptr(start), ptr(end), ptr(gaussian_ids), ptr(out),
              ptr(grad_mean), ptr(grad_cov), ptr(grad_sh_coeffs), ptr(grad_alpha), ptr(grad_out),
              ptr(topleft), ptr(c2w), int(tile_size), int(n_tiles_h), int(n_tiles_w),
              float(pixel_size_x), float(pixel_size_y), int(H), int(W), int(C), float(thresh),
              stream_handle(mean.device))


__all__ = [
    "culling_gaussian_bsphere",
    "tile_culling_aabb_start_end",
    "tile_based_vol_rendering_sh",
    "tile_based_vol_rendering_backward_sh",
]
