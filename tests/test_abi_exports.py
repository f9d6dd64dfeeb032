"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
entry point that include/gsx.h declares (no compute calls)."""
import ctypes
import re
from pathlib import Path

import pytest

from gaussian_splatting_3d_gb300 import _build, _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "gsx.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gsx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "gsx_tile_based_vol_rendering_sh" in names
    assert "gsx_tile_culling_aabb_start_end" in names
    assert len(names) >= 12


def test_library_exports_every_declared_symbol():
    path = _build.build()
    lib = ctypes.CDLL(str(path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header():
    names = set(declared_functions())
    bound = set(_lib.SIGNATURES)
    assert names <= bound | {"gsx_binning_workspace_bytes"}, names - bound


def test_status_strings_and_host_validation_without_gpu():
    lib = _lib.load()
    assert lib.gsx_abi_version() == _lib.GSX_ABI_VERSION == 3
    assert lib.gsx_status_string(0) == b"ok"
    assert lib.gsx_status_string(2) == b"capacity exceeded"
    # argument validation happens on the host before any CUDA call
    st = lib.gsx_tile_based_vol_rendering_sh(10, 10, None, None, None, None, None, None, None, None, None, None,
                                             16, 1, 1, 1.0, 1.0, 16, 16, 7, 0.01, None)
    assert st == _lib.GSX_ERR_INVALID_ARG
    assert b"SH order" in lib.gsx_last_error()
    st = lib.gsx_bin_gaussians(-1, None, None, None, 1, 1, 0, None, None, None, None, None, 0, None)
    assert st == _lib.GSX_ERR_INVALID_ARG
    assert lib.gsx_binning_workspace_bytes(1000, 4000, 64) > 4 * 4000


def test_workspace_size_grows_with_capacity():
    lib = _lib.load()
    a = lib.gsx_binning_workspace_bytes(1000, 1000, 64)
    b = lib.gsx_binning_workspace_bytes(1000, 100000, 64)
    assert b > a


def test_unaligned_binning_workspace_is_rejected_on_the_host():
    """The binning kernels read the workspace with 16-byte vector loads, so a
    workspace that does not start on a 256-byte boundary is refused before
    anything is enqueued (the pointers below are never dereferenced)."""
    lib = _lib.load()
    n, cap, ntw, nth = 1000, 4000, 8, 8
    need = lib.gsx_binning_workspace_bytes(n, cap, ntw * nth)
    fake = 1 << 40  # a non-null address; the call must return before using it
    st = lib.gsx_bin_gaussians_async(n, fake, fake, fake, ntw, nth, cap, fake, fake, fake, fake + 16, need, None)
    assert st == _lib.GSX_ERR_INVALID_ARG
    assert b"256-byte aligned" in lib.gsx_last_error()


def test_ordered_raster_entry_points_validate_on_the_host():
    """The tile-order entry points refuse missing arguments before any CUDA
    call (no GPU needed)."""
    lib = _lib.load()
    p = _lib.GsxRasterParams()
    p.width, p.height, p.tile_w, p.tile_h, p.n_tiles_w, p.n_tiles_h = 16, 16, 16, 16, 1, 1
    p.sh_order, p.sh_stride, p.pixel_size_x, p.pixel_size_y, p.T_thresh = 1, 1, 1.0, 1.0, 0.01
    fake = 1 << 40
    st = lib.gsx_render_forward_ordered(p, 1, 1, fake, fake, fake, fake, fake, fake, fake, fake, fake, fake,
                                        None, None)
    assert st == _lib.GSX_ERR_INVALID_ARG and b"tile_order" in lib.gsx_last_error()
    st = lib.gsx_render_backward_ordered(p, 1, 1, *([fake] * 15), None, None)
    assert st == _lib.GSX_ERR_INVALID_ARG and b"tile_order" in lib.gsx_last_error()
    assert lib.gsx_tile_order(None, None, -1, None, None) == _lib.GSX_ERR_INVALID_ARG
    assert lib.gsx_tile_order(None, None, 0, None, None) == _lib.GSX_OK
    assert lib.gsx_tile_order(None, None, 4, None, None) == _lib.GSX_ERR_INVALID_ARG


def declared_arities():
    """{name: parameter count} of every function declared in gsx.h."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for name, params in re.findall(r"\b(gsx_[a-z0-9_]+)\s*\(([^;{}]*?)\)\s*;", text, flags=re.S):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else len(params.split(","))
    return out


def test_ctypes_table_matches_header_arity():
    arity = declared_arities()
    assert len(arity) >= 12
    wrong = {n: (k, len(_lib.SIGNATURES[n][1])) for n, k in arity.items()
             if n in _lib.SIGNATURES and len(_lib.SIGNATURES[n][1]) != k}
    assert not wrong, f"(header, ctypes) parameter counts differ: {wrong}"


def test_training_entry_points_validate_on_the_host():
    lib = _lib.load()
    assert lib.gsx_photometric_loss_workspace_bytes(1080, 1920) == 9 * 1080 * 1920 * 4
    assert lib.gsx_photometric_loss_blocks(1080, 1920) == (3 * 1080 * 1920 + 255) // 256
    ws = ctypes.c_void_p(1)  # never dereferenced: validation fails first
    for win, h, w in ((4, 64, 64), (33, 64, 64), (11, 5, 64), (11, 64, 5)):
        st = lib.gsx_photometric_loss(ws, ws, h, w, win, ctypes.c_float(0.2), 1, ws, None, ws,
                                      1 << 30, None)
        assert st == _lib.GSX_ERR_INVALID_ARG, (win, h, w)
    assert lib.gsx_adam_step(None, None, 1, 10, None) == _lib.GSX_ERR_INVALID_ARG
    assert lib.gsx_adam_step(ws, ws, 0, 10, None) == _lib.GSX_ERR_INVALID_ARG
