"""ctypes binding of the C ABI in ``include/gsx.h`` (``_native/libgsx.so``).

The library is the product's only compute path: if it cannot be loaded, every
public call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import POINTER, c_char_p, c_float, c_int, c_int32, c_int64, c_size_t, c_uint32, c_void_p

from . import _build

GSX_ABI_VERSION = 3  # include/gsx.h
GSX_OK = 0
GSX_ERR_INVALID_ARG = 1
GSX_ERR_CAPACITY = 2
GSX_ERR_TIMEOUT = 3
GSX_ERR_CUDA = 4
GSX_ERR_MISMATCH = 5
# gradient flags of the projection backward (include/gsx.h)
GSX_GRAD_DEPTH, GSX_GRAD_JACOBIAN, GSX_GRAD_CLAMP = 1, 2, 4
GSX_GRAD_EXACT = 7


class GsxError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, func: str, detail: str):
        self.status = status
        self.func = func
        super().__init__(f"{func}: {detail or 'status ' + str(status)} (status {status})")


class GsxCapacityError(GsxError):
    pass


class GsxCamera(ctypes.Structure):
    _fields_ = [
        ("c2w", c_float * 12),
        ("fx", c_float),
        ("fy", c_float),
        ("cx", c_float),
        ("cy", c_float),
        ("width", c_int32),
        ("height", c_int32),
        ("frustum_normals", c_float * 18),
        ("frustum_pts", c_float * 18),
    ]


class GsxRasterParams(ctypes.Structure):
    _fields_ = [
        ("width", c_int32),
        ("height", c_int32),
        ("tile_w", c_int32),
        ("tile_h", c_int32),
        ("n_tiles_w", c_int32),
        ("n_tiles_h", c_int32),
        ("sh_order", c_int32),
        ("sh_stride", c_int32),
        ("pixel_size_x", c_float),
        ("pixel_size_y", c_float),
        ("T_thresh", c_float),
        ("write_empty_tiles", c_int32),
        ("pixels_per_thread", c_int32),
    ]


P = c_void_p  # device pointers and streams travel as integers

# name -> (restype, argtypes)
SIGNATURES = {
    "gsx_status_string": (c_char_p, [c_int]),
    "gsx_last_error": (c_char_p, []),
    "gsx_abi_version": (c_int, []),
    "gsx_kernel_launch_count": (ctypes.c_uint64, []),
    "gsx_culling_gaussian_bsphere": (c_int, [c_int64, P, P, P, P, P, P, c_float, P]),
    "gsx_binning_workspace_bytes": (c_size_t, [c_int64, c_int64, c_int64]),
    "gsx_tile_culling_aabb_start_end": (
        c_int,
        [c_int64, c_int64, P, P, P, c_int32, c_int32, P, P, P, P, c_size_t, P],
    ),
    "gsx_tile_culling_aabb_start_end_noalloc": (
        c_int,
        [c_int64, c_int64, P, P, P, c_int32, c_int32, P, P, P, P],
    ),
    "gsx_tile_based_vol_rendering_sh": (
        c_int,
        [c_int64, c_int64, P, P, P, P, P, P, P, P, P, P,
         c_uint32, c_uint32, c_uint32, c_float, c_float, c_uint32, c_uint32, c_uint32, c_float, P],
    ),
    "gsx_tile_based_vol_rendering_backward_sh": (
        c_int,
        [c_int64, c_int64, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P,
         c_uint32, c_uint32, c_uint32, c_float, c_float, c_uint32, c_uint32, c_uint32, c_float, P],
    ),
    "gsx_project_forward": (
        c_int,
        [c_int64, P, P, P, P, POINTER(GsxCamera), c_float, c_float, c_int32, c_int32, c_int32,
         P, P, P, P, P, P, P],
    ),
    "gsx_bin_gaussians": (
        c_int,
        [c_int64, P, P, P, c_int32, c_int32, c_int64, P, P, P, POINTER(c_int64), P, c_size_t, P],
    ),
    "gsx_bin_gaussians_async": (
        c_int,
        [c_int64, P, P, P, c_int32, c_int32, c_int64, P, P, P, P, c_size_t, P],
    ),
    "gsx_binning_status": (c_int, [P, c_int64, c_int64, c_int32, c_int32, POINTER(c_int64), P]),
    "gsx_binning_status_copy_async": (c_int, [P, c_int64, c_int64, P, P]),
    "gsx_binning_status_decode": (c_int, [P, c_int64, c_int32, c_int32, POINTER(c_int64)]),
    "gsx_render_forward": (
        c_int,
        [POINTER(GsxRasterParams), c_int64, c_int64, P, P, P, P, P, P, P, P, P, P, P],
    ),
    "gsx_tile_order": (c_int, [P, P, c_int32, P, P]),
    "gsx_project_colors": (c_int, [c_int64, P, P, c_int32, c_int32, P, P, P, P]),
    "gsx_project_colors_backward": (c_int, [c_int64, P, P, c_int32, c_int32, P, P, P, P, P, P, P]),
    "gsx_render_forward_rgb": (c_int, [POINTER(GsxRasterParams), c_int64, c_int64] + [P] * 12),
    "gsx_render_backward_rgb": (c_int, [POINTER(GsxRasterParams), c_int64, c_int64] + [P] * 17),
    "gsx_render_forward_ordered": (
        c_int,
        [POINTER(GsxRasterParams), c_int64, c_int64, P, P, P, P, P, P, P, P, P, P, P, P],
    ),
    "gsx_render_forward_maps": (
        c_int,
        [POINTER(GsxRasterParams), c_int64, c_int64, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P],
    ),
    "gsx_render_backward_ordered": (
        c_int,
        [POINTER(GsxRasterParams), c_int64, c_int64] + [P] * 17,
    ),
    "gsx_render_backward": (
        c_int,
        [POINTER(GsxRasterParams), c_int64, c_int64, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P],
    ),
    "gsx_raster_status": (c_int, [P, c_int32, P]),
    "gsx_raster_wait_selftest": (c_int, [c_uint32, P, P]),
    "gsx_exp_selftest": (c_int, [P, c_int64, P, c_int32, P]),
    "gsx_look_back_selftest_bytes": (c_size_t, []),
    "gsx_look_back_selftest": (c_int, [P, c_size_t, P, P]),
    "gsx_project_backward": (
        c_int,
        [c_int64, P, P, P, P, POINTER(GsxCamera), P, P, P, P, P, P, P, P, c_int32, P],
    ),
    # batched passes (views_dev, views_host, n_views, ...)
    "gsx_batch_view_size": (c_size_t, []),
    "gsx_batch_project_forward": (c_int, [P, P, c_int32, c_float, c_float] + [P] * 7),
    "gsx_batch_bin_async": (c_int, [P, P, c_int32, P, P, P, c_int64, P, P, P, P, c_size_t, P]),
    "gsx_batch_render_forward": (c_int, [P, P, c_int32, c_int64] + [P] * 6 + [c_float, P, P, P]),
    "gsx_batch_render_backward": (c_int, [P, P, c_int32, c_int64] + [P] * 9 + [c_float, P, P, P]),
    "gsx_batch_project_backward": (c_int, [P, P, c_int32] + [P] * 4 + [c_int32, P]),
    # adaptive density control
    "gsx_densify_count_visible": (c_int, [c_int64, P, P, P]),
    "gsx_densify_accumulate": (c_int, [c_int64, P, c_int32, P, P, c_int32, P]),
    "gsx_densify_classify": (c_int, [c_int64, P, P, P, c_float, c_float, c_int32, P, P]),
    "gsx_adam_group_size": (c_size_t, []),
    "gsx_photometric_loss_workspace_bytes": (c_size_t, [c_int32, c_int32]),
    "gsx_photometric_loss_blocks": (c_int64, [c_int32, c_int32]),
    "gsx_photometric_loss": (c_int, [P, P, c_int32, c_int32, c_int32, c_float, c_int32, P, P, P, c_size_t, P]),
    "gsx_adam_step": (c_int, [P, P, c_int32, c_int64, P]),
    "gsx_densify_rewrite": (c_int, [c_int64, P, P, P, P, c_int64, c_int64, c_int64, P, P, P, P, c_int32, P,
                                    c_float, ctypes.c_uint64, P, P, P, P, P, P]),
}

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return str(_build.LIB_PATH)


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first if needed) the native library; raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not _build.LIB_PATH.exists():
            if not build_if_missing:
                raise ImportError(f"native library missing: {_build.LIB_PATH}")
            _build.build()
        try:
            lib = ctypes.CDLL(str(_build.LIB_PATH))
        except OSError as e:
            raise ImportError(f"cannot load {_build.LIB_PATH}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.gsx_abi_version() != GSX_ABI_VERSION:
            raise ImportError(f"{_build.LIB_PATH} has ABI version {lib.gsx_abi_version()}, the bindings expect "
                              f"{GSX_ABI_VERSION}: rebuild it")
        _lib = lib
        return lib


def check(status: int, func: str) -> None:
    if status == GSX_OK:
        return
    lib = load()
    detail = (lib.gsx_last_error() or b"").decode(errors="replace")
    cls = GsxCapacityError if status == GSX_ERR_CAPACITY else GsxError
    raise cls(status, func, detail)


def call(name: str, *args) -> int:
    """Call an entry point returning a status; raise GsxError on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    check(st, name)
    return st
