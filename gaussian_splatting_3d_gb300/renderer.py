"""Differentiable rendering on the sm_103a kernels.

Two autograd entry points:

``render_sh`` -- the reference's ``_render_sh.apply`` (gs/renderer.py:672-828)
    with the same 18 positional arguments, running the raster forward and
    backward through this package's ``_gs`` functions.

``rasterize`` / ``FusedRender`` -- the fused native path behind ``SHRenderer``:
    projection (cull + EWA covariance + AABB count, one kernel), deterministic
    tile binning, raster forward; backward = raster backward + projection
    backward (parity mode: depth detached and J constant, exactly the
    derivative the reference's autograd takes, gs/renderer.py:365-419).  The
    projection is recomputed in the backward from the parameters, so only the
    2D record (mean2d, cov2d, alpha), the key lists and the image are kept
    between the passes.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _gs, _lib
from ._lib import GsxRasterParams
from ._torch import check_tensor, ptr, stream_handle
from .camera import CameraInfo, make_gsx_camera


class _render_sh(torch.autograd.Function):
    """Mirror of gs/renderer.py:672-828 on the drop-in ``_gs`` functions."""

    @staticmethod
    def forward(ctx, mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, topleft, c2w, tile_size,
                n_tiles_h, n_tiles_w, pixel_size_x, pixel_size_y, H, W, C, thresh):
        out = torch.zeros([H * W * 3], dtype=torch.float32, device=mean.device)
        _gs.tile_based_vol_rendering_sh(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out,
                                        topleft, c2w, tile_size, n_tiles_h, n_tiles_w, pixel_size_x,
                                        pixel_size_y, H, W, C, thresh)
        ctx.save_for_backward(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out, topleft, c2w)
        ctx.const = [tile_size, n_tiles_h, n_tiles_w, pixel_size_x, pixel_size_y, H, W, C, thresh]
        return out

    @staticmethod
    def backward(ctx, grad):
        mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out, topleft, c2w = ctx.saved_tensors
        grad_mean = torch.zeros_like(mean)
        grad_cov = torch.zeros_like(cov)
        grad_sh_coeffs = torch.zeros_like(sh_coeffs)
        grad_alpha = torch.zeros_like(alpha)
        _gs.tile_based_vol_rendering_backward_sh(mean, cov, sh_coeffs, alpha, start, end, gaussian_ids,
                                                 out, grad_mean, grad_cov, grad_sh_coeffs, grad_alpha,
                                                 grad.contiguous(), topleft, c2w, *ctx.const)
        return (grad_mean, grad_cov, grad_sh_coeffs, grad_alpha) + (None,) * 14


render_sh = _render_sh.apply


@dataclass
class RasterSettings:
    """Renderer options with the reference's defaults (conf/garden_sh.yaml:19-36)."""

    tile_w: int = 16
    tile_h: int = 16
    frustum_culling_radius: float = 1.0
    tile_culling_radius: float = 6.0
    T_thresh: float = 0.01
    sh_order: int | None = None  # C used for colour (now_C); None = all coefficients
    # gradient semantics: the reference detaches depth in mean2d (depth_detach,
    # gs/sh_renderer.py:144), builds J without gradient and ignores the opacity
    # clamp; exact_grad=True gives the true derivative of the image
    depth_detach: bool = True
    exact_grad: bool = False
    # memory mode: hold only the tile lists between forward and backward (the
    # projection is re-run in backward, bit-identically; the binning workspace
    # is released after each forward)
    recompute_projection: bool = False
    # background colour composited behind the Gaussians (None: black, as the
    # reference's default bg=False) and per-pixel alpha / depth maps
    bg: tuple | None = None
    output_maps: bool = False
    # "pixel": SH evaluated per pixel from the pixel's ray (the reference);
    # "gaussian": one colour per Gaussian per view from the direction camera
    # centre -> mean, computed once in the projection (opt-in, not the
    # reference's images)
    sh_mode: str = "pixel"
    # per-pixel SH direction: "reference" reads the [3,4] camera-to-world with
    # a row stride of 3, as the reference does (vol_render_sh.h:48-65);
    # "ray" uses the true ray direction R (x, y, 1) (opt-in, not the
    # reference's images)
    sh_dir: str = "reference"
    # raster schedule: pixels per thread (1, or 2 for tiles made of 8x8
    # blocks; 0 = one for the forward and two for the backward, the faster
    # measured choice); images are identical and gradients agree within
    # rounding, the choice is a matter of speed
    pixels_per_thread: int = 0

    def grad_flags(self) -> int:
        if self.exact_grad:
            return _lib.GSX_GRAD_EXACT
        return 0 if self.depth_detach else _lib.GSX_GRAD_DEPTH

    def tiles(self, cam: CameraInfo):
        return (cam.w + self.tile_w - 1) // self.tile_w, (cam.h + self.tile_h - 1) // self.tile_h


class BinningBuffers:
    """Reusable device buffers for the key lists of one device (grow-only)."""

    def __init__(self, device: torch.device):
        self.device = device
        self.capacity = 0
        self.n = -1
        self.ws = None
        self.ids = None

    def ensure(self, n: int, capacity: int, n_tiles: int):
        if capacity > self.capacity or n != self.n or self.ws is None:
            cap = max(capacity, self.capacity)
            ws_bytes = _lib.load().gsx_binning_workspace_bytes(n, cap, n_tiles)
            self.ws = torch.empty(ws_bytes, dtype=torch.uint8, device=self.device)
            self.ids = torch.empty(max(cap, 1), dtype=torch.int32, device=self.device)
            self.capacity = cap
            self.n = n
        return self

    def release(self):
        self.ws = None
        self.ids = None
        self.capacity = 0
        self.n = -1


_buffers: dict = {}


def _bin_buffers(device) -> BinningBuffers:
    key = (device.type, device.index)
    if key not in _buffers:
        _buffers[key] = BinningBuffers(device)
    return _buffers[key]


@dataclass
class Projected:
    mean2d: torch.Tensor
    cov2d: torch.Tensor
    depth: torch.Tensor
    alpha: torch.Tensor
    rect: torch.Tensor
    counts: torch.Tensor


def project(mean, qvec, log_scale, alpha_logit, gcam, settings: RasterSettings,
            scales_are_activated: bool = False) -> Projected:
    n = mean.shape[0]
    dev = mean.device
    pr = Projected(
        torch.empty((n, 2), dtype=torch.float32, device=dev),
        torch.empty((n, 4), dtype=torch.float32, device=dev),
        torch.empty((n,), dtype=torch.float32, device=dev),
        torch.empty((n,), dtype=torch.float32, device=dev),
        torch.empty((n, 4), dtype=torch.int32, device=dev),
        torch.empty((n,), dtype=torch.int32, device=dev),
    )
    _lib.call("gsx_project_forward", n, ptr(mean), ptr(qvec), ptr(log_scale), ptr(alpha_logit),
              ctypes.byref(gcam), float(settings.frustum_culling_radius), float(settings.tile_culling_radius),
              int(settings.tile_w), int(settings.tile_h), int(bool(scales_are_activated)), ptr(pr.mean2d),
              ptr(pr.cov2d), ptr(pr.depth), ptr(pr.alpha), ptr(pr.rect), ptr(pr.counts), stream_handle(dev))
    return pr


def bin_gaussians(pr: Projected, n_tiles_w: int, n_tiles_h: int, key_hint: int | None = None):
    """Sorted Gaussian ids per tile (synchronising): returns (ids[K], start[T], end[T], K)."""
    n = pr.counts.shape[0]
    dev = pr.counts.device
    T = n_tiles_w * n_tiles_h
    buf = _bin_buffers(dev)
    cap = max(buf.capacity, key_hint or 0, 4 * n, 1 << 16)
    start = torch.empty((T,), dtype=torch.int32, device=dev)
    end = torch.empty((T,), dtype=torch.int32, device=dev)
    for _ in range(3):
        buf.ensure(n, cap, T)
        k = ctypes.c_int64(0)
        st = _lib.load().gsx_bin_gaussians(n, ptr(pr.rect), ptr(pr.counts), ptr(pr.depth), n_tiles_w, n_tiles_h,
                                           buf.capacity, ptr(buf.ids), ptr(start), ptr(end), ctypes.byref(k),
                                           ptr(buf.ws), buf.ws.numel(), stream_handle(dev))
        if st == _lib.GSX_ERR_CAPACITY and k.value > buf.capacity:
            cap = int(k.value * 1.25) + 1024
            continue
        _lib.check(st, "gsx_bin_gaussians")
        K = int(k.value)
        return buf.ids[:K].clone() if K > 0 else buf.ids[:0].clone(), start, end, K
    raise _lib.GsxCapacityError(_lib.GSX_ERR_CAPACITY, "gsx_bin_gaussians", "could not size the key buffer")


def bin_gaussians_async(pr: Projected, n_tiles_w: int, n_tiles_h: int, capacity: int):
    """Enqueue the binning without synchronising: returns (ids[capacity],
    start, end); binning_status() later gives the key count (it synchronises
    the stream), or binning_status_async() + decode_binning_status() without
    waiting for work enqueued after the binning."""
    n = pr.counts.shape[0]
    dev = pr.counts.device
    T = n_tiles_w * n_tiles_h
    buf = _bin_buffers(dev).ensure(n, capacity, T)
    ids = torch.empty((max(capacity, 1),), dtype=torch.int32, device=dev)
    start = torch.empty((T,), dtype=torch.int32, device=dev)
    end = torch.empty((T,), dtype=torch.int32, device=dev)
    _lib.call("gsx_bin_gaussians_async", n, ptr(pr.rect), ptr(pr.counts), ptr(pr.depth), n_tiles_w, n_tiles_h,
              capacity, ptr(ids), ptr(start), ptr(end), ptr(buf.ws), buf.ws.numel(), stream_handle(dev))
    return ids, start, end


def binning_status(dev, n: int, capacity: int, n_tiles_w: int, n_tiles_h: int):
    """(status, key count) of the last asynchronous binning on `dev` (synchronises)."""
    buf = _bin_buffers(dev)
    k = ctypes.c_int64(0)
    st = _lib.load().gsx_binning_status(ptr(buf.ws), n, capacity, n_tiles_w, n_tiles_h, ctypes.byref(k),
                                        stream_handle(dev))
    return st, int(k.value)


def binning_status_async(dev, n: int, capacity: int, block: torch.Tensor) -> torch.cuda.Event:
    """Enqueue on the current stream a copy of the last binning's 16-byte
    status block into `block` (16 bytes of pinned host memory) and return an
    event: after event.synchronize(), decode_binning_status(block, ...) gives
    what binning_status would.  Work enqueued after this call does not delay
    the event, so a caller can launch the raster first and wait only for the
    binning."""
    buf = _bin_buffers(dev)
    _lib.check(_lib.load().gsx_binning_status_copy_async(ptr(buf.ws), n, capacity, block.data_ptr(),
                                                         stream_handle(dev)), "gsx_binning_status_copy_async")
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(dev))
    return ev


def decode_binning_status(block: torch.Tensor, capacity: int, n_tiles_w: int, n_tiles_h: int):
    """(status, key count) from a status block that has arrived."""
    k = ctypes.c_int64(0)
    st = _lib.load().gsx_binning_status_decode(block.data_ptr(), capacity, n_tiles_w, n_tiles_h, ctypes.byref(k))
    return st, int(k.value)


def raster_status(dev=None, clear: bool = True) -> int:
    """Sticky error bits of the raster kernels on `dev` (synchronises; 0 =
    no error).  Bit 0: a wait for the bulk copies of a batch's SH rows gave
    up, so some tile's output or gradients are incomplete."""
    dev = torch.device(dev) if dev is not None else torch.device("cuda", torch.cuda.current_device())
    flags = ctypes.c_uint32(0)
    with torch.cuda.device(dev):
        _lib.call("gsx_raster_status", ctypes.addressof(flags), 1 if clear else 0, stream_handle(dev))
    return int(flags.value)


def _raster_params(cam: CameraInfo, settings: RasterSettings, C: int, sh_stride: int) -> GsxRasterParams:
    ntw, nth = settings.tiles(cam)
    p = GsxRasterParams()
    p.width, p.height = int(cam.w), int(cam.h)
    p.tile_w, p.tile_h = int(settings.tile_w), int(settings.tile_h)
    p.n_tiles_w, p.n_tiles_h = int(ntw), int(nth)
    p.sh_order, p.sh_stride = int(C), int(sh_stride)
    p.pixel_size_x, p.pixel_size_y = float(1.0 / cam.fx), float(1.0 / cam.fy)
    p.T_thresh = float(settings.T_thresh)
    p.write_empty_tiles = 1
    p.pixels_per_thread = int(settings.pixels_per_thread)
    return p


def camera_floats(c2w_np, cam: CameraInfo, sh_dir: str = "reference") -> np.ndarray:
    """float32 [14]: the image-plane top-left corner (2 floats) and the 12
    camera floats the raster reads for the per-pixel SH direction (rows of 3
    at float offsets 0, 3, 6).  "reference": the row-major [3,4]
    camera-to-world as is, so the direction uses its misread rows as the
    reference does; "ray": the rotation's rows packed contiguously, so the
    same reads give the ray direction R (x, y, 1)."""
    if sh_dir not in ("reference", "ray"):
        raise ValueError(f"sh_dir must be 'reference' or 'ray' (got {sh_dir!r})")
    m = np.ascontiguousarray(c2w_np, dtype=np.float32).reshape(3, 4)
    flat = m.reshape(12) if sh_dir == "reference" else np.concatenate([m[:, :3].reshape(9), m[:, 3]])
    return np.concatenate([np.asarray(cam.topleft(), np.float32), flat]).astype(np.float32)


def camera_consts(c2w_np, cam: CameraInfo, sh_dir: str = "reference") -> torch.Tensor:
    """camera_floats in a pinned host tensor (uploaded without blocking)."""
    t = torch.empty(14, dtype=torch.float32, pin_memory=True)
    t.copy_(torch.from_numpy(camera_floats(c2w_np, cam, sh_dir)))
    return t


class ViewPipeline:
    """One view through the fused native path with persistent device buffers.

    ``forward`` runs projection, binning and the raster forward and returns a
    state object; ``backward`` runs the raster backward and the projection
    backward from dL/dimage.  When ``timer`` is given, CUDA events bracket
    each stage on the launching stream (names: project, binning, raster_fwd,
    raster_bwd, project_bwd)."""

    def __init__(self, device=None):
        self.device = torch.device(device or "cuda")
        self.key_capacity = 0  # grows to ~1.25x the largest key count seen
        self.status_block = None  # pinned 16 bytes: the binning's status, read without a stream sync

    def forward(self, mean, qvec, log_scale, sh, alpha_logit, c2w_np, cam: CameraInfo,
                settings: RasterSettings, timer=None, sh_ready=None, cam_consts=None,
                prepare_grads: bool = False):
        """``sh_ready``: an event the raster stage waits for (the SH
        coefficients still arriving on a copy stream while projection and
        binning run); ``cam_consts``: the device copy of
        ``camera_consts(c2w_np, cam)`` when the caller uploaded it;
        ``prepare_grads``: a backward will follow, so its zeroed gradient
        accumulators are filled on a side stream while the raster forward
        runs (not in the memory mode, which holds nothing extra between the
        passes)."""
        dev = mean.device
        n = mean.shape[0]
        sh_stride = sh.shape[-1]
        C = settings.sh_order or int(round(sh_stride ** 0.5))
        rgb_mode = settings.sh_mode == "gaussian"
        if settings.sh_mode not in ("pixel", "gaussian"):
            raise ValueError(f"sh_mode must be 'pixel' or 'gaussian' (got {settings.sh_mode!r})")
        if rgb_mode and (settings.bg is not None or settings.output_maps):
            raise NotImplementedError("per-Gaussian colours composite no background and write no maps")
        gcam = make_gsx_camera(c2w_np, cam)
        ev = timer.stage if timer is not None else (lambda name: _null_ctx())
        with ev("project"):
            pr = project(mean, qvec, log_scale, alpha_logit, gcam, settings)
        ntw, nth = settings.tiles(cam)
        if cam_consts is None:
            cam_consts = camera_consts(c2w_np, cam, settings.sh_dir).to(dev, non_blocking=True)
        topleft, c2w_dev = cam_consts[:2], cam_consts[2:]
        out = torch.empty((cam.h, cam.w, 3), dtype=torch.float32, device=dev)
        order = torch.empty((ntw * nth,), dtype=torch.int32, device=dev)
        params = _raster_params(cam, settings, C, sh_stride)
        grads = grads_ready = None
        rgb = None
        cam_pos = (ctypes.c_float * 3)(*[float(v) for v in np.asarray(c2w_np, np.float32).reshape(3, 4)[:, 3]])
        cap = max(self.key_capacity, 1 << 16)
        want_grads = prepare_grads and not settings.recompute_projection
        for _ in range(3):
            with ev("binning"):
                ids, start, end = bin_gaussians_async(pr, ntw, nth, cap)
            # the key count comes back without waiting for the raster enqueued
            # below, so this call returns while the raster forward runs
            if self.status_block is None:
                self.status_block = torch.zeros(16, dtype=torch.uint8, pin_memory=True)
            status_ev = binning_status_async(dev, n, cap, self.status_block)
            if want_grads and grads is None:
                binned = torch.cuda.Event()
                binned.record(torch.cuda.current_stream(dev))
            if sh_ready is not None:  # only the raster reads the SH coefficients
                torch.cuda.current_stream(dev).wait_event(sh_ready)
            if rgb_mode and rgb is None:
                with ev("colors"):
                    rgb = torch.empty((n, 3), dtype=torch.float32, device=dev)
                    _lib.call("gsx_project_colors", n, ptr(mean), ptr(sh), sh_stride, C, ctypes.addressof(cam_pos),
                              ptr(pr.counts), ptr(rgb), stream_handle(dev))
            with ev("raster_fwd"):
                if rgb_mode:
                    _lib.call("gsx_tile_order", ptr(start), ptr(end), ntw * nth, ptr(order), stream_handle(dev))
                    _lib.call("gsx_render_forward_rgb", ctypes.byref(params), n, cap, ptr(pr.mean2d), ptr(pr.cov2d),
                              ptr(rgb), ptr(pr.alpha), ptr(start), ptr(end), ptr(ids), ptr(topleft), ptr(c2w_dev),
                              ptr(out), ptr(order), stream_handle(dev))
                elif settings.bg is None and not settings.output_maps:
                    # longest tile lists first: the order changes the schedule, not the image
                    _lib.call("gsx_tile_order", ptr(start), ptr(end), ntw * nth, ptr(order), stream_handle(dev))
                    _lib.call("gsx_render_forward_ordered", ctypes.byref(params), n, cap, ptr(pr.mean2d),
                              ptr(pr.cov2d), ptr(sh), ptr(pr.alpha), ptr(start), ptr(end), ptr(ids), ptr(topleft),
                              ptr(c2w_dev), ptr(out), ptr(order), stream_handle(dev))
                else:
                    bg = (ctypes.c_float * 3)(*settings.bg) if settings.bg is not None else None
                    if settings.output_maps:
                        maps = (torch.empty((cam.h, cam.w), dtype=torch.float32, device=dev),
                                torch.empty((cam.h, cam.w), dtype=torch.float32, device=dev))
                    _lib.call("gsx_render_forward_maps", ctypes.byref(params), n, cap, ptr(pr.mean2d),
                              ptr(pr.cov2d), ptr(sh), ptr(pr.alpha), ptr(start), ptr(end), ptr(ids), ptr(topleft),
                              ptr(c2w_dev), ptr(out), ctypes.addressof(bg) if bg is not None else None,
                              ptr(pr.depth), ptr(maps[0]) if settings.output_maps else None,
                              ptr(maps[1]) if settings.output_maps else None, stream_handle(dev))
            if want_grads and grads is None:
                # set up after the raster launch (host time off the GPU's critical path); the
                # fill itself starts after the binning, whose working set lives in L2
                grads, grads_ready = _zeroed_grad_buffers(dev, n, (n, 3) if rgb_mode else tuple(sh.shape), binned)
            status_ev.synchronize()
            st, K = decode_binning_status(self.status_block, cap, ntw, nth)
            if st == _lib.GSX_ERR_CAPACITY:
                cap = int(K * 1.25) + 4096
                self.key_capacity = cap
                continue
            _lib.check(st, "gsx_bin_gaussians_async")
            break
        else:
            raise _lib.GsxCapacityError(_lib.GSX_ERR_CAPACITY, "binning", "could not size the key buffer")
        # keep the capacity near 1.25 K so the sort grids stay small
        if K * 2 < self.key_capacity:
            self.key_capacity = max(int(K * 1.25) + 4096, 1 << 16)
        visible_counts = pr.counts
        if settings.recompute_projection:
            visible_counts = pr.counts.clone()
            pr = None
            _bin_buffers(dev).release()
        st = dict(pr=pr, ids=ids, start=start, end=end, K=K, cap=cap, topleft=topleft, c2w_dev=c2w_dev,
                  order=order if settings.bg is None and not settings.output_maps else None,
                  rgb=rgb, cam_pos=cam_pos, C=C,
                  out=out, params=params, gcam=gcam, grad_flags=settings.grad_flags(), settings=settings,
                  counts=visible_counts)
        if settings.output_maps:
            st["alpha_map"], st["depth_map"] = maps
        if grads is not None:
            st["grads"], st["grads_ready"] = grads, grads_ready
        return st

    def backward(self, state, mean, qvec, log_scale, sh, alpha_logit, grad_out, timer=None, sh_grad_sink=None):
        dev = mean.device
        n = mean.shape[0]
        pr = state["pr"]
        ev = timer.stage if timer is not None else (lambda name: _null_ctx())
        if pr is None:  # memory mode: the same projection again (deterministic, bit-identical)
            with ev("project_recompute"):
                pr = project(mean, qvec, log_scale, alpha_logit, state["gcam"], state["settings"])
        grad_out = grad_out.contiguous()
        rgb = state.get("rgb")
        acc_shape = (n, 3) if rgb is not None else tuple(sh.shape)  # dL/drgb or dL/dsh accumulator
        if state.get("grads") is not None and tuple(state["grads"][3].shape) == acc_shape:
            torch.cuda.current_stream(dev).wait_event(state["grads_ready"])
            g_mean2d, g_cov2d, g_alpha, g_acc = state.pop("grads")
        else:
            g_mean2d = torch.zeros((n, 2), dtype=torch.float32, device=dev)
            g_cov2d = torch.zeros((n, 4), dtype=torch.float32, device=dev)
            g_alpha = torch.zeros((n,), dtype=torch.float32, device=dev)
            g_acc = torch.zeros(acc_shape, dtype=torch.float32, device=dev)
        with ev("raster_bwd"):
            common = (ctypes.byref(state["params"]), n, state["cap"], ptr(pr.mean2d), ptr(pr.cov2d),
                      ptr(rgb if rgb is not None else sh), ptr(pr.alpha), ptr(state["start"]), ptr(state["end"]),
                      ptr(state["ids"]), ptr(state["topleft"]), ptr(state["c2w_dev"]), ptr(state["out"]),
                      ptr(grad_out), ptr(g_mean2d), ptr(g_cov2d), ptr(g_acc), ptr(g_alpha))
            if rgb is not None:
                _lib.call("gsx_render_backward_rgb", *common, ptr(state["order"]), stream_handle(dev))
            elif state.get("order") is not None:  # the forward's order (longest lists first)
                _lib.call("gsx_render_backward_ordered", *common, ptr(state["order"]), stream_handle(dev))
            else:
                _lib.call("gsx_render_backward", *common, stream_handle(dev))
        if sh_grad_sink is not None and rgb is None:
            sh_grad_sink(g_acc)  # dL/dsh is final here: the projection backward does not touch it
        g_mean = torch.empty_like(mean)
        g_q = torch.empty_like(qvec)
        g_ls = torch.empty_like(log_scale)
        g_al = torch.empty_like(alpha_logit)
        with ev("project_bwd"):
            _lib.call("gsx_project_backward", n, ptr(mean), ptr(qvec), ptr(log_scale), ptr(alpha_logit),
                      ctypes.byref(state["gcam"]), ptr(pr.counts), ptr(g_mean2d), ptr(g_cov2d), ptr(g_alpha),
                      ptr(g_mean), ptr(g_q), ptr(g_ls), ptr(g_al), state["grad_flags"], stream_handle(dev))
        if rgb is not None:  # dL/drgb -> dL/dsh, and the view direction's share of dL/dmean
            g_sh = torch.empty_like(sh)
            with ev("colors_bwd"):
                _lib.call("gsx_project_colors_backward", n, ptr(mean), ptr(sh), sh.shape[-1], state["C"],
                          ctypes.addressof(state["cam_pos"]), ptr(pr.counts), ptr(rgb), ptr(g_acc), ptr(g_sh),
                          ptr(g_mean), stream_handle(dev))
        else:
            g_sh = g_acc
        state["g_mean2d"] = g_mean2d  # dL/dmean2d (normalised image coordinates), for densification
        return g_mean, g_q, g_ls, g_sh, g_al


class _null_ctx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


class StageTimer:
    """CUDA events around pipeline stages on the current stream; durations
    are read after a synchronize."""

    def __init__(self):
        self.records = []  # (name, start_event, end_event)

    def stage(self, name):
        timer = self

        class _Ctx:
            def __enter__(self):
                self.s = torch.cuda.Event(enable_timing=True)
                self.e = torch.cuda.Event(enable_timing=True)
                self.s.record()
                return self

            def __exit__(self, *a):
                self.e.record()
                timer.records.append((name, self.s, self.e))
                return False

        return _Ctx()

    def summary(self):
        torch.cuda.synchronize()
        out = {}
        for name, s, e in self.records:
            out.setdefault(name, []).append(s.elapsed_time(e))
        return {k: dict(mean_ms=float(np.mean(v)), count=len(v)) for k, v in out.items()}


_pipelines: dict = {}


def _pipeline(device) -> ViewPipeline:
    key = (device.type, device.index)
    if key not in _pipelines:
        _pipelines[key] = ViewPipeline(device)
    return _pipelines[key]


_copy_streams: dict = {}
_fill_streams: dict = {}


def _zeroed_grad_buffers(device, n: int, acc_shape: tuple, after: torch.cuda.Event):
    """The raster backward's accumulators (dL/dmean2d [n,2], dL/dcov2d [n,4],
    dL/dalpha [n], and dL/dsh or dL/drgb of shape acc_shape), zero-filled on a
    side stream that starts at `after` (an event of the current stream
    recorded before any kernel that uses memory these fresh blocks may have
    held); returns them and the event the backward waits for."""
    main = torch.cuda.current_stream(device)
    key = (device.type, device.index)
    if key not in _fill_streams:
        _fill_streams[key] = torch.cuda.Stream(device)
    fs = _fill_streams[key]
    bufs = (torch.empty((n, 2), dtype=torch.float32, device=device),
            torch.empty((n, 4), dtype=torch.float32, device=device),
            torch.empty((n,), dtype=torch.float32, device=device),
            torch.empty(acc_shape, dtype=torch.float32, device=device))
    fs.wait_event(after)
    done = torch.cuda.Event()
    with torch.cuda.stream(fs):
        for b in bufs:
            b.zero_()
            b.record_stream(fs)
        done.record(fs)
    return bufs, done


def copy_stream(device) -> torch.cuda.Stream:
    """The stream on which host-resident ``rasterize`` uploads the parameters
    of `device`.  A caller's further host->device copies for the same step
    (e.g. the loss weights) enqueued here after the call land behind the
    parameters instead of sharing the link with them, so the SH coefficients
    the raster waits for arrive first."""
    device = torch.device(device)
    key = (device.type, device.index)
    if key not in _copy_streams:
        _copy_streams[key] = torch.cuda.Stream(device)
    return _copy_streams[key]


_d2h_streams: dict = {}


def _d2h_stream(device) -> torch.cuda.Stream:
    key = (device.type, device.index)
    if key not in _d2h_streams:
        _d2h_streams[key] = torch.cuda.Stream(device)
    return _d2h_streams[key]


def _upload_overlapped(host, consts, device):
    """Copy the camera constants and the host parameters (mean, qvec,
    log_scale, sh, alpha_logit) to `device` on a copy stream: constants and
    the four geometry tensors first, then the SH coefficients.  The current
    stream waits only for the first group, so projection and binning run
    while the SH coefficients (the bulk of the bytes) are still in flight;
    nothing else is copied host->device before the raster, so no copy on the
    current stream queues behind them.  Returns the device tensors, the
    device constants and the event the raster stage must wait for."""
    main = torch.cuda.current_stream(device)
    cs = copy_stream(device)
    dev_t = [torch.empty(h.shape, dtype=h.dtype, device=device) for h in host]
    dev_c = torch.empty(consts.shape, dtype=consts.dtype, device=device)
    cs.wait_stream(main)  # the fresh buffers may reuse memory the main stream still reads
    geo_done = torch.cuda.Event()
    sh_done = torch.cuda.Event()
    with torch.cuda.stream(cs):
        for d, h in [(dev_c, consts)] + [(dev_t[k], host[k]) for k in (0, 1, 2, 4, 3)]:
            d.copy_(h, non_blocking=True)
            d.record_stream(cs)
            if d is dev_t[4]:
                geo_done.record(cs)
        sh_done.record(cs)
    main.wait_event(geo_done)
    return dev_t, dev_c, sh_done


class FusedRender(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mean, qvec, log_scale, sh, alpha_logit, c2w_np, cam, settings, aux=None, device=None):
        host_mode = not mean.is_cuda
        names = ("mean", "qvec", "log_scale", "sh_coeffs", "alpha_logit")
        tensors = (mean, qvec, log_scale, sh, alpha_logit)
        sh_ready = cam_consts = None
        if host_mode:
            # host-resident parameters: uploaded every call, overlapped with
            # projection and binning; gradients come back to the host
            for x, name in zip(tensors, names):
                check_tensor(x, name, cuda=False)
                if x.is_cuda:
                    raise RuntimeError(f"{name} must be on the host like mean")
            dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
            with torch.cuda.device(dev):
                (mean, qvec, log_scale, sh, alpha_logit), cam_consts, sh_ready = _upload_overlapped(
                    tensors, camera_consts(c2w_np, cam, settings.sh_dir), dev)
        else:
            for x, name in zip(tensors, names):
                check_tensor(x, name)
        pipe = _pipeline(mean.device)
        with torch.cuda.device(mean.device):
            state = pipe.forward(mean, qvec, log_scale, sh, alpha_logit, c2w_np, cam, settings, sh_ready=sh_ready,
                                 cam_consts=cam_consts, prepare_grads=any(ctx.needs_input_grad[:5]))
        ctx.save_for_backward(mean, qvec, log_scale, sh, alpha_logit)
        ctx.host_mode = host_mode
        ctx.state = state
        ctx.pipe = pipe
        ctx.aux = aux
        if aux is not None:  # per-Gaussian key counts of this view (0 = culled), optional maps
            aux["counts"] = state["counts"]
            if "alpha_map" in state:
                aux["alpha_map"], aux["depth_map"] = state["alpha_map"], state["depth_map"]
        return state["out"]

    @staticmethod
    def backward(ctx, grad_out):
        mean, qvec, log_scale, sh, alpha_logit = ctx.saved_tensors
        dev = mean.device
        with torch.cuda.device(dev):
            if not ctx.host_mode:
                grads = ctx.pipe.backward(ctx.state, mean, qvec, log_scale, sh, alpha_logit, grad_out)
            else:
                # gradients of host parameters live on the host.  dL/dsh (the
                # bulk of the bytes) starts its download on a side stream as
                # soon as the raster backward has produced it, overlapping the
                # projection backward; the other four follow.
                main = torch.cuda.current_stream(dev)
                d2h = _d2h_stream(dev)
                sh_host = []

                def sink(g):
                    h = torch.empty(g.shape, dtype=g.dtype, pin_memory=True)
                    d2h.wait_stream(main)
                    with torch.cuda.stream(d2h):
                        h.copy_(g, non_blocking=True)
                    g.record_stream(d2h)
                    sh_host.append(h)

                grads = ctx.pipe.backward(ctx.state, mean, qvec, log_scale, sh, alpha_logit, grad_out,
                                          sh_grad_sink=sink)
                host = []
                for k, g in enumerate(grads):
                    if k == 3 and sh_host:
                        host.append(sh_host[0])
                        continue
                    h = torch.empty(g.shape, dtype=g.dtype, pin_memory=True)
                    h.copy_(g, non_blocking=True)
                    host.append(h)
                main.synchronize()
                d2h.synchronize()
                grads = tuple(host)
        if ctx.aux is not None:
            ctx.aux["mean2d_grad"] = ctx.state["g_mean2d"]
        ctx.state = None
        return grads + (None, None, None, None, None)


def rasterize(mean, qvec, log_scale, sh_coeffs, alpha_logit, c2w, cam: CameraInfo,
              settings: RasterSettings | None = None, aux: dict | None = None, device=None) -> torch.Tensor:
    """Render one view: parameters as in SHRenderer (log-scales, opacity
    logits, SH [N,3,C_max^2]) and a [3,4] camera-to-world (host array or
    tensor).  Returns the [H,W,3] image; differentiable w.r.t. all five
    parameter tensors.  With an ``aux`` dict, the forward stores the
    per-Gaussian key counts (``aux["counts"]``, 0 = culled) and the backward
    dL/dmean2d (``aux["mean2d_grad"]``, [N,2]) for adaptive density control;
    with ``settings.output_maps`` also the alpha (1 - final transmittance) and
    depth (sum of T a G z) maps (``aux["alpha_map"]``, ``aux["depth_map"]``,
    [H,W], not differentiated).  ``settings.bg`` composites a background
    colour behind the Gaussians (the gradients include it).

    Host-resident parameters (CPU tensors, pinned for overlap) are uploaded
    to ``device`` (default: the current CUDA device) on every call, the SH
    coefficients overlapped with projection and binning; the image is
    returned on the device and the backward returns the parameters'
    gradients on the host (pinned)."""
    settings = settings or RasterSettings()
    if isinstance(c2w, torch.Tensor):
        c2w = c2w.detach().to("cpu", torch.float32).numpy()
    return FusedRender.apply(mean, qvec, log_scale, sh_coeffs, alpha_logit, np.asarray(c2w, np.float32), cam,
                             settings, aux, device)
