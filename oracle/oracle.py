"""TEST INFRASTRUCTURE ONLY: numpy/ctypes wrapper of the C oracle
(oracle/gsx_oracle.c).  Imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py -- never by the product package.

Builds ``oracle/_build/liboracle.so`` with gcc (-O2 -fopenmp
-ffp-contract=off) on first use.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
from ctypes import POINTER, c_float, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "gsx_oracle.c"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

MIN_RENDER_ALPHA = np.float32(1.0) / np.float32(255.0)


def build(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    stamp = BUILD / "liboracle.sha256"
    fp = hashlib.sha256(SRC.read_bytes()).hexdigest()
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return LIB
    tmp = BUILD / "liboracle.so.tmp"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp), str(SRC), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(fp)
    return LIB


class OrcCamera(ctypes.Structure):
    _fields_ = [
        ("c2w", c_float * 12),
        ("fx", c_float), ("fy", c_float), ("cx", c_float), ("cy", c_float),
        ("width", c_int32), ("height", c_int32),
        ("normals", c_float * 18),
        ("pts", c_float * 18),
    ]


class OrcRasterParams(ctypes.Structure):
    _fields_ = [
        ("width", c_int32), ("height", c_int32), ("tile_w", c_int32), ("tile_h", c_int32),
        ("n_tiles_w", c_int32), ("n_tiles_h", c_int32), ("C", c_int32), ("sh_stride", c_int32),
        ("T_thresh", c_float),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        _lib.orc_expf.restype = c_float
        _lib.orc_expf.argtypes = [c_float]
        _lib.orc_bin.restype = c_int64
        _lib.orc_num_threads.restype = c_int32
    return _lib


def _p(a):
    return a.ctypes.data_as(c_void_p) if a is not None else None


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def expf(x: float) -> np.float32:
    return np.float32(lib().orc_expf(float(x)))


def make_camera(c2w, fx, fy, cx, cy, width, height, normals, pts) -> OrcCamera:
    c = OrcCamera()
    c.c2w[:] = [float(v) for v in f32(c2w).reshape(-1)]
    c.fx, c.fy, c.cx, c.cy = float(fx), float(fy), float(cx), float(cy)
    c.width, c.height = int(width), int(height)
    c.normals[:] = [float(v) for v in f32(normals).reshape(-1)]
    c.pts[:] = [float(v) for v in f32(pts).reshape(-1)]
    return c


def cull_bsphere(mean, svec, normals, pts, thresh):
    mean, svec = f32(mean), f32(svec)
    n = mean.shape[0]
    mask = np.zeros(n, dtype=np.uint8)
    lib().orc_cull_bsphere(c_int64(n), _p(mean), _p(svec), _p(f32(normals)), _p(f32(pts)), c_float(thresh),
                           _p(mask))
    return mask.astype(bool)


def project(mean, qvec, log_s, alpha_logit, cam: OrcCamera, frustum_radius=1.0, tile_radius=6.0,
            tile_w=16, tile_h=16, scales_are_svec=False):
    mean, qvec, log_s = f32(mean), f32(qvec), f32(log_s)
    n = mean.shape[0]
    out = dict(
        mask=np.zeros(n, np.uint8), mean2d=np.zeros((n, 2), np.float32), cov2d=np.zeros((n, 4), np.float32),
        depth=np.zeros(n, np.float32), alpha=np.zeros(n, np.float32), rect=np.zeros((n, 4), np.int32),
        counts=np.zeros(n, np.int32),
    )
    al = f32(alpha_logit) if alpha_logit is not None else None
    lib().orc_project(c_int64(n), _p(mean), _p(qvec), _p(log_s), _p(al), ctypes.byref(cam),
                      c_float(frustum_radius), c_float(tile_radius), c_int32(tile_w), c_int32(tile_h),
                      c_int32(int(scales_are_svec)), _p(out["mask"]), _p(out["mean2d"]), _p(out["cov2d"]),
                      _p(out["depth"]), _p(out["alpha"]), _p(out["rect"]), _p(out["counts"]))
    out["mask"] = out["mask"].astype(bool)
    return out


def bin_gaussians(tl, br, depth, n_tiles_h, n_tiles_w, stride=2, want_keys=False):
    """tl/br: [n,2] int32 (stride 2) or one packed [n,4] array passed as both
    (tl=rect, br=rect[:,2:], stride 4)."""
    depth = f32(depth).reshape(-1)
    n = depth.shape[0]
    T = n_tiles_h * n_tiles_w
    start = np.zeros(T, np.int32)
    end = np.zeros(T, np.int32)
    if stride == 4:
        rect = i32(tl)
        tl_p = rect.ctypes.data_as(c_void_p)
        br_p = c_void_p(rect.ctypes.data + 8)
        keep = rect
    else:
        tl, br = i32(tl), i32(br)
        tl_p, br_p = _p(tl), _p(br)
        keep = (tl, br)
    K = int(lib().orc_bin(c_int64(n), tl_p, br_p, c_int32(stride), _p(depth), c_int32(n_tiles_h),
                          c_int32(n_tiles_w), c_int64(0), None, None, _p(start), _p(end)))
    # second call with the exact capacity
    ids = np.zeros(max(K, 1), np.int32)
    keys = np.zeros(max(K, 1), np.uint64) if want_keys else None
    K2 = int(lib().orc_bin(c_int64(n), tl_p, br_p, c_int32(stride), _p(depth), c_int32(n_tiles_h),
                           c_int32(n_tiles_w), c_int64(K), _p(ids), _p(keys), _p(start), _p(end)))
    del keep
    assert K2 == K
    res = dict(ids=ids[:K], start=start, end=end, K=K)
    if want_keys:
        res["keys"] = keys[:K]
    return res


def raster_params(width, height, tile_w, tile_h, C, sh_stride=None, T_thresh=0.01):
    p = OrcRasterParams()
    p.width, p.height, p.tile_w, p.tile_h = int(width), int(height), int(tile_w), int(tile_h)
    p.n_tiles_w = (int(width) + tile_w - 1) // tile_w
    p.n_tiles_h = (int(height) + tile_h - 1) // tile_h
    p.C = int(C)
    p.sh_stride = int(sh_stride if sh_stride is not None else C * C)
    p.T_thresh = float(T_thresh)
    return p


def render_fwd(P: OrcRasterParams, mean2d, cov2d, sh, alpha, start, end, ids, topleft, c2w, psx, psy,
               bg=None, depth=None, maps: bool = False):
    """Image [H,W,3]; with maps=True also (alpha map, depth map) [H,W] (depth
    needs the per-Gaussian depth).  bg: background RGB composited behind."""
    out = np.zeros((P.height, P.width, 3), np.float32)
    am = np.zeros((P.height, P.width), np.float32) if maps else None
    dm = np.zeros((P.height, P.width), np.float32) if maps and depth is not None else None
    bgv = f32(np.asarray(bg, np.float32)) if bg is not None else None
    lib().orc_render_fwd_ex(ctypes.byref(P), _p(f32(mean2d)), _p(f32(cov2d)), _p(f32(sh)), _p(f32(alpha)),
                            _p(i32(start)), _p(i32(end)), _p(i32(ids)), _p(f32(topleft)), _p(f32(c2w)),
                            c_float(psx), c_float(psy), _p(out), _p(bgv) if bgv is not None else None,
                            _p(f32(depth)) if dm is not None else None, _p(am) if am is not None else None,
                            _p(dm) if dm is not None else None)
    return (out, am, dm) if maps else out


def render_bwd(P: OrcRasterParams, mean2d, cov2d, sh, alpha, start, end, ids, topleft, c2w, psx, psy, out,
               grad_out):
    mean2d, cov2d, sh, alpha = f32(mean2d), f32(cov2d), f32(sh), f32(alpha)
    n = alpha.shape[0]
    g = dict(mean2d=np.zeros((n, 2), np.float32), cov2d=np.zeros((n, 4), np.float32),
             sh=np.zeros_like(sh), alpha=np.zeros(n, np.float32))
    lib().orc_render_bwd(ctypes.byref(P), _p(mean2d), _p(cov2d), _p(sh), _p(alpha), _p(i32(start)), _p(i32(end)),
                         _p(i32(ids)), _p(f32(topleft)), _p(f32(c2w)), c_float(psx), c_float(psy), _p(f32(out)),
                         _p(f32(grad_out)), _p(g["mean2d"]), _p(g["cov2d"]), _p(g["sh"]), _p(g["alpha"]))
    return g


GRAD_DEPTH, GRAD_JACOBIAN, GRAD_CLAMP = 1, 2, 4
GRAD_EXACT = GRAD_DEPTH | GRAD_JACOBIAN | GRAD_CLAMP


def project_bwd(mean, qvec, log_s, alpha_logit, cam: OrcCamera, mask, g_mean2d, g_cov2d, g_alpha, flags: int = 0):
    """flags = 0: the reference's gradient (depth detached, J constant, opacity
    clamp ignored); GRAD_* bits add the true-derivative terms."""
    mean, qvec, log_s, alpha_logit = f32(mean), f32(qvec), f32(log_s), f32(alpha_logit)
    n = mean.shape[0]
    out = dict(mean=np.zeros((n, 3), np.float32), qvec=np.zeros((n, 4), np.float32),
               log_scale=np.zeros((n, 3), np.float32), alpha_logit=np.zeros(n, np.float32))
    m = np.ascontiguousarray(mask, dtype=np.uint8)
    lib().orc_project_bwd(c_int64(n), _p(mean), _p(qvec), _p(log_s), _p(alpha_logit), ctypes.byref(cam), _p(m),
                          _p(f32(g_mean2d)), _p(f32(g_cov2d)), _p(f32(g_alpha)), _p(out["mean"]), _p(out["qvec"]),
                          _p(out["log_scale"]), _p(out["alpha_logit"]), ctypes.c_int32(flags))
    return out


def num_threads() -> int:
    return int(lib().orc_num_threads())


def render_view(scene, view, grad_weight=None, frustum_radius=1.0, tile_radius=6.0, T_thresh=0.01,
                sh_order=None, grad_flags: int = 0, bg=None):
    """Full oracle pipeline for one view of a scene.Scene / scene.View:
    project, bin, raster forward and (if grad_weight is given) backward
    through the projection.  Returns a dict of every intermediate."""
    from gaussian_splatting_3d_gb300.camera import frustum_np  # host math only (numpy/torch CPU)

    cam = view.cam
    normals, pts = frustum_np(view.c2w, cam)
    ocam = make_camera(view.c2w, cam.fx, cam.fy, cam.cx, cam.cy, cam.w, cam.h, normals, pts)
    pr = project(scene.mean, scene.qvec, scene.log_scale, scene.alpha_logit, ocam, frustum_radius, tile_radius,
                 view.tile, view.tile)
    ntw = (cam.w + view.tile - 1) // view.tile
    nth = (cam.h + view.tile - 1) // view.tile
    b = bin_gaussians(pr["rect"], pr["rect"][:, 2:], pr["depth"], nth, ntw, stride=4)
    C = sh_order or scene.sh_order
    P = raster_params(cam.w, cam.h, view.tile, view.tile, C, scene.sh.shape[-1], T_thresh)
    topleft = np.array(cam.topleft(), np.float32)
    psx, psy = np.float32(1.0 / cam.fx), np.float32(1.0 / cam.fy)
    img, am, dm = render_fwd(P, pr["mean2d"], pr["cov2d"], scene.sh, pr["alpha"], b["start"], b["end"], b["ids"],
                             topleft, view.c2w, psx, psy, bg=bg, depth=pr["depth"], maps=True)
    res = dict(proj=pr, bins=b, image=img, alpha_map=am, depth_map=dm, camera=ocam, params=P, topleft=topleft)
    if grad_weight is not None:
        g = render_bwd(P, pr["mean2d"], pr["cov2d"], scene.sh, pr["alpha"], b["start"], b["end"], b["ids"],
                       topleft, view.c2w, psx, psy, img, grad_weight)
        gp = project_bwd(scene.mean, scene.qvec, scene.log_scale, scene.alpha_logit, ocam, pr["mask"],
                         g["mean2d"], g["cov2d"], g["alpha"], grad_flags)
        res["raster_grads"] = g
        res["param_grads"] = dict(gp, sh=g["sh"])
    return res
