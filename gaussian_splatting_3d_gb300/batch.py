"""Multi-view batching: many cameras (any mix of image sizes, one or several
resident scenes) rendered with ONE launch per stage, optionally replayed as a
captured CUDA graph.

A batch is planned once (``BatchPipeline.plan``): the (view, Gaussian) items
and the tiles of all views are numbered consecutively, every per-item and
per-tile buffer is allocated up front, and the view table is uploaded to the
device.  A step is then projection -> binning -> raster forward
(-> raster backward -> projection backward) over the whole batch, with no host
synchronisation; the key count is checked once afterwards and the step is
re-run with a larger key capacity if it did not fit.  Because the buffers are
static the step can be captured in a CUDA graph and replayed.

Images are identical to rendering each view alone with the same tile shape:
per tile, the sorted list and the per-pixel arithmetic are the same.
"""
from __future__ import annotations

import ctypes
from ctypes import c_float, c_int32, c_int64, c_void_p
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import GsxCamera
from ._torch import check_tensor, ptr, stream_handle
from .camera import CameraInfo, make_gsx_camera
from .renderer import RasterSettings


class GsxBatchView(ctypes.Structure):
    _fields_ = [
        ("mean", c_void_p), ("qvec", c_void_p), ("log_scale", c_void_p), ("alpha_logit", c_void_p),
        ("sh", c_void_p),
        ("g_mean", c_void_p), ("g_qvec", c_void_p), ("g_log_scale", c_void_p), ("g_alpha_logit", c_void_p),
        ("g_sh", c_void_p),
        ("n_gaussians", c_int64), ("item_offset", c_int64), ("tile_offset", c_int64),
        ("sh_stride", c_int32), ("sh_order", c_int32),
        ("tile_w", c_int32), ("tile_h", c_int32), ("n_tiles_w", c_int32), ("n_tiles_h", c_int32),
        ("topleft", c_float * 2), ("pixel_size_x", c_float), ("pixel_size_y", c_float),
        ("out", c_void_p), ("grad_out", c_void_p),
        ("write_empty_tiles", c_int32), ("pixels_per_thread", c_int32),
        ("cam", GsxCamera),
    ]


def _lib_batch():
    lib = _lib.load()
    if lib.gsx_batch_view_size() != ctypes.sizeof(GsxBatchView):
        raise ImportError(f"gsx_batch_view layout mismatch: library {lib.gsx_batch_view_size()} bytes, "
                          f"binding {ctypes.sizeof(GsxBatchView)} bytes")
    return lib


@dataclass
class Scene:
    """Device-resident parameters of one scene (as SHRenderer holds them)."""

    mean: torch.Tensor
    qvec: torch.Tensor
    log_scale: torch.Tensor
    sh: torch.Tensor
    alpha_logit: torch.Tensor

    @property
    def n(self) -> int:
        return int(self.mean.shape[0])

    @classmethod
    def from_checkpoint(cls, path, device) -> "Scene":
        """A scene from an SHRenderer checkpoint (gs/sh_renderer.py:663-679)."""
        from .checkpoint import load_state

        sd = load_state(path, device)
        return cls(sd["mean"], sd["qvec"], sd["svec_before_activation"], sd["sh_coeffs"],
                   sd["alpha_before_activation"])

    @classmethod
    def from_arrays(cls, sc, device) -> "Scene":
        return cls(*(torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in
                     (sc.mean, sc.qvec, sc.log_scale, sc.sh, sc.alpha_logit)))


@dataclass
class ViewSpec:
    scene: int          # index into the batch's scene list
    c2w: np.ndarray     # [3,4]
    cam: CameraInfo


class BatchPipeline:
    """Plan once, then step (eager or graph replay) over a fixed set of views."""

    def __init__(self, device=None, settings: RasterSettings | None = None, persistent: bool = True):
        """persistent: the raster passes run as persistent grids that claim
        the batch's tiles longest list first (gsx_tile_order + a work
        counter); False launches one CTA per tile in index order.  Neither
        choice changes an image or a gradient."""
        self.device = torch.device(device or "cuda")
        self.settings = settings or RasterSettings()
        self.persistent = persistent
        self.graph = None
        self.key_capacity = 0

    # ------------------------------------------------------------------ plan
    def plan(self, scenes: list[Scene], views: list[ViewSpec], backward: bool = True, sh_order: int | None = None):
        dev = self.device
        st = self.settings
        if st.bg is not None or st.output_maps:
            raise NotImplementedError("batched passes composite no background and write no maps")
        if st.sh_mode != "pixel" or st.sh_dir != "reference":
            raise NotImplementedError("batched passes use the reference's per-pixel SH colour")
        self.scenes = scenes
        self.views = views
        self.backward_enabled = backward
        V = len(views)
        used = {v.scene for v in views}
        if any(scenes[i] is None for i in used):
            raise ValueError("a view refers to a scene that is not resident")
        C = sh_order or st.sh_order or int(round(scenes[views[0].scene].sh.shape[-1] ** 0.5))
        self.C = C
        for s in (scenes[i] for i in sorted(used)):
            for t, name in ((s.mean, "mean"), (s.qvec, "qvec"), (s.log_scale, "log_scale"), (s.sh, "sh"),
                            (s.alpha_logit, "alpha_logit")):
                check_tensor(t, name)
        if backward and len(scenes) != 1:
            raise ValueError("the batched backward needs all views to share one scene")
        table = (GsxBatchView * V)()
        item, tile = 0, 0
        pix_offsets = []
        total_pix = 0
        for i, v in enumerate(views):
            ntw, nth = st.tiles(v.cam)
            pix_offsets.append(total_pix)
            total_pix += v.cam.w * v.cam.h * 3
        self.image_flat = torch.zeros(total_pix, dtype=torch.float32, device=dev)
        self.images = [self.image_flat[o:o + v.cam.w * v.cam.h * 3].view(v.cam.h, v.cam.w, 3)
                       for o, v in zip(pix_offsets, views)]
        if backward:
            self.grad_out_flat = torch.zeros(total_pix, dtype=torch.float32, device=dev)
            self.grad_outs = [self.grad_out_flat[o:o + v.cam.w * v.cam.h * 3].view(v.cam.h, v.cam.w, 3)
                              for o, v in zip(pix_offsets, views)]
            s0 = scenes[0]
            self.g_mean = torch.zeros_like(s0.mean)
            self.g_qvec = torch.zeros_like(s0.qvec)
            self.g_log_scale = torch.zeros_like(s0.log_scale)
            self.g_alpha_logit = torch.zeros_like(s0.alpha_logit)
            self.g_sh = torch.zeros_like(s0.sh)
        for i, v in enumerate(views):
            sc = scenes[v.scene]
            ntw, nth = st.tiles(v.cam)
            e = table[i]
            e.mean, e.qvec, e.log_scale, e.alpha_logit, e.sh = (ptr(sc.mean), ptr(sc.qvec), ptr(sc.log_scale),
                                                               ptr(sc.alpha_logit), ptr(sc.sh))
            if backward:
                e.g_mean, e.g_qvec, e.g_log_scale, e.g_alpha_logit, e.g_sh = (
                    ptr(self.g_mean), ptr(self.g_qvec), ptr(self.g_log_scale), ptr(self.g_alpha_logit),
                    ptr(self.g_sh))
                e.grad_out = ptr(self.grad_outs[i])
            e.n_gaussians = sc.n
            e.item_offset = item
            e.tile_offset = tile
            e.sh_stride = int(sc.sh.shape[-1])
            e.sh_order = C
            e.tile_w, e.tile_h = st.tile_w, st.tile_h
            e.n_tiles_w, e.n_tiles_h = ntw, nth
            tl = v.cam.topleft()
            e.topleft[0], e.topleft[1] = float(tl[0]), float(tl[1])
            e.pixel_size_x, e.pixel_size_y = float(1.0 / v.cam.fx), float(1.0 / v.cam.fy)
            e.out = ptr(self.images[i])
            e.write_empty_tiles = 1
            e.pixels_per_thread = int(st.pixels_per_thread)
            e.cam = make_gsx_camera(v.c2w, v.cam)
            item += sc.n
            tile += ntw * nth
        self.n_items, self.n_tiles = item, tile
        self.table = table
        raw = torch.frombuffer(bytearray(bytes(table)), dtype=torch.uint8)
        self._table_pinned = raw.pin_memory()  # kept alive until the copy has run
        self.table_dev = self._table_pinned.to(dev, non_blocking=True)
        I = item
        f32 = dict(dtype=torch.float32, device=dev)
        self.mean2d = torch.empty((I, 2), **f32)
        self.cov2d = torch.empty((I, 4), **f32)
        self.depth = torch.empty((I,), **f32)
        self.alpha = torch.empty((I,), **f32)
        self.rect = torch.empty((I, 4), dtype=torch.int32, device=dev)
        self.counts = torch.empty((I,), dtype=torch.int32, device=dev)
        self.start = torch.empty((tile,), dtype=torch.int32, device=dev)
        self.end = torch.empty((tile,), dtype=torch.int32, device=dev)
        self.order = torch.empty((tile,), dtype=torch.int32, device=dev)
        self.work_counter = torch.zeros((4,), dtype=torch.int32, device=dev)
        if backward:
            self.g_mean2d = torch.zeros((I, 2), **f32)
            self.g_cov2d = torch.zeros((I, 4), **f32)
            self.g_alpha = torch.zeros((I,), **f32)
        # a capacity set before planning is kept (callers that size it themselves)
        self._alloc_keys(self.key_capacity if self.key_capacity > 0 else max(4 * I, 1 << 16))
        self.graph = None
        return self

    def _alloc_keys(self, cap: int):
        lib = _lib.load()
        self.key_capacity = int(cap)
        self.ws_bytes = lib.gsx_binning_workspace_bytes(self.n_items, self.key_capacity, self.n_tiles)
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        self.ids = torch.empty((max(self.key_capacity, 1),), dtype=torch.int32, device=self.device)
        self.graph = None

    # ------------------------------------------------------------- stages
    def _views_args(self):
        return ptr(self.table_dev), ctypes.addressof(self.table), len(self.views)

    def _queue_args(self):
        """(tile_order, work_counter) of the raster passes: the order written
        after the binning by forward_async, or none for index order."""
        if not self.persistent:
            return None, None
        return ptr(self.order), ptr(self.work_counter)

    def forward_async(self):
        lib = _lib_batch()
        vd, vh, V = self._views_args()
        s = stream_handle(self.device)
        st = self.settings
        _lib.check(lib.gsx_batch_project_forward(vd, vh, V, float(st.frustum_culling_radius),
                                                 float(st.tile_culling_radius), ptr(self.mean2d), ptr(self.cov2d),
                                                 ptr(self.depth), ptr(self.alpha), ptr(self.rect), ptr(self.counts),
                                                 s), "gsx_batch_project_forward")
        _lib.check(lib.gsx_batch_bin_async(vd, vh, V, ptr(self.rect), ptr(self.counts), ptr(self.depth),
                                           self.key_capacity, ptr(self.ids), ptr(self.start), ptr(self.end),
                                           ptr(self.ws), self.ws_bytes, s), "gsx_batch_bin_async")
        if self.persistent:
            _lib.check(lib.gsx_tile_order(ptr(self.start), ptr(self.end), self.n_tiles, ptr(self.order), s),
                       "gsx_tile_order")
        _lib.check(lib.gsx_batch_render_forward(vd, vh, V, self.key_capacity, ptr(self.mean2d), ptr(self.cov2d),
                                                ptr(self.alpha), ptr(self.start), ptr(self.end), ptr(self.ids),
                                                float(st.T_thresh), *self._queue_args(), s),
                   "gsx_batch_render_forward")

    def backward_async(self):
        lib = _lib_batch()
        vd, vh, V = self._views_args()
        s = stream_handle(self.device)
        self.g_mean2d.zero_()
        self.g_cov2d.zero_()
        self.g_alpha.zero_()
        self.g_sh.zero_()
        _lib.check(lib.gsx_batch_render_backward(vd, vh, V, self.key_capacity, ptr(self.mean2d), ptr(self.cov2d),
                                                 ptr(self.alpha), ptr(self.start), ptr(self.end), ptr(self.ids),
                                                 ptr(self.g_mean2d), ptr(self.g_cov2d), ptr(self.g_alpha),
                                                 float(self.settings.T_thresh), *self._queue_args(), s),
                   "gsx_batch_render_backward")
        _lib.check(lib.gsx_batch_project_backward(vd, vh, V, ptr(self.counts), ptr(self.g_mean2d),
                                                  ptr(self.g_cov2d), ptr(self.g_alpha),
                                                  self.settings.grad_flags(), s),
                   "gsx_batch_project_backward")

    def key_status(self):
        """(status, key count) of the last binning (synchronises)."""
        k = ctypes.c_int64(0)
        st = _lib.load().gsx_binning_status(ptr(self.ws), self.n_items, self.key_capacity, 0, 0, ctypes.byref(k),
                                            stream_handle(self.device))
        return st, int(k.value)

    def _run(self, fn):
        for _ in range(4):
            fn()
            st, K = self.key_status()
            if st == _lib.GSX_ERR_CAPACITY:
                self._alloc_keys(int(K * 1.25) + 4096)
                continue
            _lib.check(st, "batched binning")
            self.n_keys = K
            return K
        raise _lib.GsxCapacityError(_lib.GSX_ERR_CAPACITY, "batched binning", "could not size the key buffer")

    def step(self):
        """Eager forward (+ backward): images in self.images, gradients in self.g_*."""
        def fn():
            self.forward_async()
            if self.backward_enabled:
                self.backward_async()
        return self._run(fn)

    def forward(self):
        return self._run(self.forward_async)

    # ------------------------------------------------------------- graphs
    def capture(self):
        """Capture one step in a CUDA graph (after an eager step has sized the
        key buffers); replay() re-runs it."""
        self.step()
        self._alloc_keys(max(self.key_capacity, int(self.n_keys * 1.25) + 4096))
        self.step()  # warm-up with the final buffers (sets kernel attributes outside capture)
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.forward_async()
                if self.backward_enabled:
                    self.backward_async()
        torch.cuda.current_stream(self.device).wait_stream(s)
        self.graph = g
        return g

    def replay(self, check: bool = True):
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()
        if check:
            st, K = self.key_status()
            if st == _lib.GSX_ERR_CAPACITY:  # scene changed: grow, recapture, redo
                self._alloc_keys(int(K * 1.25) + 4096)
                self.capture()
                return self.replay(check)
            _lib.check(st, "batched binning")
            self.n_keys = K
        return self.n_keys if check else None


def autotune_tile(scenes, views, shapes=((8, 8), (16, 16), (32, 8)), base: RasterSettings | None = None,
                  backward: bool = True, reps: int = 3, device=None, schedules=(0, 1, 2)):
    """Time one batched step per tile shape and raster schedule (pixels per
    thread: 0 = one in the forward and two in the backward, 1, 2) and return
    (best (tile_w, tile_h, pixels_per_thread), {that key: ms}).  The tile
    shape changes the AABB tile rectangles and therefore the images: record
    the choice and keep it fixed when comparing runs.  The schedule changes
    no image (and the gradients only within rounding)."""
    base = base or RasterSettings()
    times = {}
    for tw, th in shapes:
        bp = None
        for ppt in schedules:
            if ppt == 2 and (tw % 8 or th % 8):
                continue  # two pixels per thread needs tiles made of 8x8 blocks
            st = RasterSettings(**{**base.__dict__, "tile_w": tw, "tile_h": th, "pixels_per_thread": ppt})
            bp = BatchPipeline(device, st).plan(scenes, views, backward)
            bp.step()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                bp.step()
            e1.record()
            torch.cuda.synchronize()
            times[(tw, th, ppt)] = e0.elapsed_time(e1) / reps
            del bp
    best = min(times, key=times.get)
    return best, times
