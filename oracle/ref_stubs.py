"""TEST INFRASTRUCTURE: what importing the reference's Python
needs in an environment without its third-party dependencies.

``install_stubs()`` puts inert stand-ins for cv2, matplotlib, torchtyping,
faiss (and rich and tqdm, where they are not installed) into ``sys.modules`` (imported by the reference, unused on the render
path) and restates kornia's ``quaternion_to_rotation_matrix`` from its
published math (normalise q, then the WXYZ rotation matrix;
utils/transforms.py:31-45 calls it).  ``reference_cfg`` is the renderer
configuration of conf/garden_sh.yaml:19-46 as the reference's SHRenderer
reads it.
"""
from __future__ import annotations

import sys
import types

import torch


def install_stubs(cpu_only: bool = False):
    def mod(name, **attrs):
        m = types.ModuleType(name)
        m.__dict__.update(attrs)
        sys.modules[name] = m
        return m

    mod("cv2")
    try:  # present here, absent on the GPU hosts
        import rich.console  # noqa: F401
    except ImportError:
        class Console:
            def __init__(self, *a, **k):
                pass

            def print(self, *a, **k):
                pass

            log = print

        mod("rich").console = mod("rich.console", Console=Console)
    try:
        import tqdm  # noqa: F401
    except ImportError:
        mod("tqdm", tqdm=lambda it=None, *a, **k: it)
    mpl = mod("matplotlib")
    mpl.pyplot = mod("matplotlib.pyplot")
    mod("faiss")

    class _TT:
        def __class_getitem__(cls, item):
            return torch.Tensor

    mod("torchtyping", TensorType=_TT)

    class QuaternionCoeffOrder:
        XYZW = "xyzw"
        WXYZ = "wxyz"

    def quaternion_to_rotation_matrix(quaternion, order=QuaternionCoeffOrder.WXYZ):
        q = torch.nn.functional.normalize(quaternion, p=2.0, dim=-1, eps=1e-12)
        if order == QuaternionCoeffOrder.XYZW:
            x, y, z, w = torch.chunk(q, chunks=4, dim=-1)
        else:
            w, x, y, z = torch.chunk(q, chunks=4, dim=-1)
        tx, ty, tz = 2.0 * x, 2.0 * y, 2.0 * z
        twx, twy, twz = tx * w, ty * w, tz * w
        txx, txy, txz = tx * x, ty * x, tz * x
        tyy, tyz, tzz = ty * y, tz * y, tz * z
        one = torch.tensor(1.0)
        m = torch.stack([one - (tyy + tzz), txy - twz, txz + twy,
                         txy + twz, one - (txx + tzz), tyz - twx,
                         txz - twy, tyz + twx, one - (txx + tyy)], dim=-1)
        return m.view(quaternion.shape[:-1] + (3, 3))

    def rotation_matrix_to_quaternion(*a, **k):  # imported, never called on this path
        raise NotImplementedError

    conv = mod("kornia.geometry.conversions", QuaternionCoeffOrder=QuaternionCoeffOrder,
               quaternion_to_rotation_matrix=quaternion_to_rotation_matrix,
               rotation_matrix_to_quaternion=rotation_matrix_to_quaternion)
    geo = mod("kornia.geometry", conversions=conv)
    mod("kornia", geometry=geo)

    class _Cudart:
        def cudaProfilerStart(self):
            return 0

        def cudaProfilerStop(self):
            return 0

    if cpu_only:  # torch without CUDA: the reference's profiler hooks become no-ops
        torch.cuda.profiler.cudart = lambda: _Cudart()


class Cfg(dict):
    __getattr__ = dict.__getitem__


def reference_cfg(C_max: int, tile: int, device: str = "cpu") -> Cfg:
    # renderer keys as in conf/garden_sh.yaml:19-46; training keys are unused here
    return Cfg(device=device, sh_order=C_max, svec_act="exp", alpha_act="sigmoid", tile_size=tile,
               near_plane=1.5, far_plane=1000.0, frustum_culling_radius=1.0, tile_culling_type="aabb",
               tile_culling_thresh=0.01, tile_culling_radius=6.0, T_thresh=0.01, sh_upgrades=[2000, 4000],
               adaptive_control_iteration=800, pos_grad_thresh=0.0002, split_scale_thresh=0.02,
               scale_shrink_factor=1.6, alpha_reset_period=100000000, remove_low_alpha_period=10000000,
               alpha_reset_val=0.1, alpha_thresh=0.05, max_iteration=10000, mean_lr=1e-3, qvec_lr=1e-2,
               svec_lr=1e-2, sh_coeffs_lr=1e-2, alpha_lr=1e-2, warmup_steps=0, debug=False)
