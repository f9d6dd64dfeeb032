"""Pinhole camera of the reference (utils/camera.py:219-314) and the camera
record handed to the native projection.

``CameraInfo`` keeps the reference's fields and methods, so code written
against it (``get_frustum``, ``camera_space_to_pixel_space``,
``from_fov_camera``) runs unchanged.  Coordinates are normalised image-plane
coordinates: pixel (px, py) sits at ``topleft + (px, py) / (fx, fy)`` with
``topleft = (-cx/fx, -cy/fy)`` (gs/sh_renderer.py:242-248).
"""
from __future__ import annotations

import math
from collections import OrderedDict

import numpy as np
import torch
import torch.nn.functional as F

from ._lib import GsxCamera


class CameraInfo:
    """Intrinsics, image size and near/far planes (utils/camera.py:219-247)."""

    def __init__(self, fx, fy, cx, cy, w, h, near_plane, far_plane) -> None:
        self.fx, self.fy = fx, fy
        self.cx, self.cy = cx, cy
        self.w, self.h = w, h
        self.yfov = 2 * np.arctan(self.h / (2 * self.fy))
        self.aspect = w / h
        self.near_plane = near_plane
        self.far_plane = far_plane

    def downsample(self, scale):
        self.fx /= scale
        self.fy /= scale
        self.cx /= scale
        self.cy /= scale
        self.w //= scale
        self.h //= scale
        self.yfov = 2 * np.arctan(self.h / (2 * self.fy))
        self.aspect = self.w / self.h

    def upsample(self, scale):
        self.fx *= scale
        self.fy *= scale
        self.cx *= scale
        self.cy *= scale
        self.w *= int(scale)
        self.h *= int(scale)

    def get_frustum(self, c2w: torch.Tensor):
        """Six frustum half-spaces (normals normalised, points) for a [3,4] c2w,
        with the reference's plane construction (utils/camera.py:249-283)."""
        up = -c2w[:, 1]
        right = c2w[:, 0]
        lookat = c2w[:, 2]
        t = c2w[:, 3]
        half_vside = float(self.far_plane * np.tan(self.yfov * 0.5))
        half_hside = half_vside * float(self.aspect)
        near_point = float(self.near_plane) * lookat
        far_point = float(self.far_plane) * lookat
        near_normal = lookat
        far_normal = -lookat
        left_normal = torch.linalg.cross(far_point - half_hside * right, up)
        right_normal = torch.linalg.cross(up, far_point + half_hside * right)
        up_normal = torch.linalg.cross(far_point + half_vside * up, right)
        down_normal = torch.linalg.cross(right, far_point - half_vside * up)
        pts = torch.stack([near_point + t, far_point + t, t, t, t, t], dim=0)
        normals = torch.stack(
            [near_normal, far_normal, left_normal, right_normal, up_normal, down_normal], dim=0
        )
        normals = F.normalize(normals, dim=-1)
        return normals, pts

    def camera_space_to_pixel_space(self, pts):
        """Normalised coordinates to int32 pixels (utils/camera.py:290-303)."""
        if pts.shape[1] == 3:
            pts = pts[:, :2] / pts[:, 2:]
        assert pts.shape[1] == 2
        pts[:, 0] = pts[:, 0] * self.fx + self.cx
        pts[:, 1] = pts[:, 1] * self.fy + self.cy
        if isinstance(pts, np.ndarray):
            pts = pts.astype(np.int32)
        elif isinstance(pts, torch.Tensor):
            pts = pts.to(torch.int32)
        return pts

    @classmethod
    def from_fov_camera(cls, fov, aspect, resolution, near_plane, far_plane):
        """FoV applied per axis, as the reference viewer does (utils/camera.py:305-314)."""
        W = resolution
        H = int(resolution / aspect)
        cx = W / 2
        cy = H / 2
        fx = cx / np.tan(fov / 2)
        fy = cy / np.tan(fov / 2)
        return cls(fx, fy, cx, cy, W, H, near_plane, far_plane)

    @classmethod
    def from_vertical_fov(cls, fov_deg, width, height, near_plane=1.5, far_plane=1000.0):
        """Square pixels, vertical FoV: fx = fy = (H/2)/tan(fov/2), principal point at the centre."""
        f = (height / 2.0) / math.tan(math.radians(fov_deg) / 2.0)
        return cls(f, f, width / 2.0, height / 2.0, width, height, near_plane, far_plane)

    def topleft(self):
        return (-self.cx / self.fx, -self.cy / self.fy)


def look_at_c2w(pos, look_at=(0.0, 0.0, 0.0), up=None) -> np.ndarray:
    """[3,4] camera-to-world with columns (x, y, z, position), z towards
    ``look_at`` and y = -up, as gs/debug.py:23-37 builds it; x is normalised
    so the rotation stays orthonormal when ``up`` is not perpendicular to z.
    ``up`` defaults to +z, or +y when the view direction is within 8 degrees of z."""
    pos = np.asarray(pos, dtype=np.float64)
    z = np.asarray(look_at, dtype=np.float64) - pos
    z = z / np.linalg.norm(z)
    if up is None:
        up = np.array([0.0, 0.0, 1.0])
        if abs(float(np.dot(z, up))) > 0.99:
            up = np.array([0.0, 1.0, 0.0])
    up = np.asarray(up, dtype=np.float64)
    up = up / np.linalg.norm(up)
    y = -up
    x = np.cross(y, z)
    x = x / np.linalg.norm(x)
    y = np.cross(z, x)
    c2w = np.zeros((3, 4), dtype=np.float32)
    c2w[:, 0] = x
    c2w[:, 1] = y
    c2w[:, 2] = z
    c2w[:, 3] = pos
    return c2w


def frustum_np(c2w: np.ndarray, cam: CameraInfo):
    """get_frustum evaluated in float32 on the host; returns (normals, pts) [6,3]."""
    n, p = cam.get_frustum(torch.from_numpy(np.ascontiguousarray(c2w, dtype=np.float32)))
    return n.numpy().astype(np.float32), p.numpy().astype(np.float32)


_CAMERA_CACHE: "OrderedDict[tuple, GsxCamera]" = OrderedDict()
_CAMERA_CACHE_SIZE = 256


def make_gsx_camera(c2w: np.ndarray, cam: CameraInfo) -> GsxCamera:
    """Camera record of the native projection (c2w, intrinsics, image size,
    frustum half-spaces).  The frustum costs ~0.2 ms of small torch CPU ops,
    so records are memoised on the exact camera (c2w bits and every
    CameraInfo field); callers must not modify the returned record."""
    c2w = np.ascontiguousarray(c2w, dtype=np.float32).reshape(3, 4)
    key = (c2w.tobytes(), float(cam.fx), float(cam.fy), float(cam.cx), float(cam.cy), int(cam.w), int(cam.h),
           float(cam.yfov), float(cam.aspect), float(cam.near_plane), float(cam.far_plane))
    g = _CAMERA_CACHE.get(key)
    if g is not None:
        _CAMERA_CACHE.move_to_end(key)
        return g
    normals, pts = frustum_np(c2w, cam)
    g = GsxCamera()
    g.c2w[:] = [float(v) for v in c2w.reshape(-1)]
    g.fx, g.fy, g.cx, g.cy = float(cam.fx), float(cam.fy), float(cam.cx), float(cam.cy)
    g.width, g.height = int(cam.w), int(cam.h)
    g.frustum_normals[:] = [float(v) for v in normals.reshape(-1)]
    g.frustum_pts[:] = [float(v) for v in pts.reshape(-1)]
    _CAMERA_CACHE[key] = g
    if len(_CAMERA_CACHE) > _CAMERA_CACHE_SIZE:
        _CAMERA_CACHE.popitem(last=False)
    return g
