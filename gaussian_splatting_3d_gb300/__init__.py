"""GB300-native (sm_103a) differentiable SH Gaussian-splatting rasteriser.

A drop-in replacement for the CUDA extension ``_gs`` of heheyas/gaussian_splatting_3d
(module :mod:`gaussian_splatting_3d_gb300._gs`) plus a fused native path
(:mod:`gaussian_splatting_3d_gb300.renderer`) behind the reference's
``SHRenderer`` call surface (:mod:`gaussian_splatting_3d_gb300.sh_renderer`).
All compute runs in hand-written CUDA kernels in ``_native/libgsx.so``; there
is no CPU fallback.
"""
from ._lib import GsxCapacityError, GsxError  # noqa: F401

__all__ = ["GsxError", "GsxCapacityError"]
