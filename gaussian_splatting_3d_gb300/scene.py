"""Seeded synthetic scenes and cameras for the benchmark workloads.

Random numbers come from numpy's PCG64 bit generator (its raw stream is
stable across numpy versions and platforms) keyed by (seed, stream id);
uniforms take the top 53 bits, normals use Box-Muller in float64 and are
rounded once to float32, so the same seed gives the same float32 scene on the
x86 build host and on the Arm GPU host.

Workloads (sizes and distributions as specified for the path's benchmarks):
  * ``small``: 10,000 Gaussians, means U[-1,1]^3, log-scales N(-3, 0.5),
    quaternions normalise(N(0,1)^4), opacity logits N(0,1), SH degree 0 with
    RGB U[0,1] encoded as logit(rgb)/Y00; camera at (0,0,-4) looking at the
    origin, 60 deg vertical FoV, 256x256, 16x16 tiles.
  * ``headline``: 1,000,000 Gaussians, means N(0, 2^2) clipped to |x| <= 6,
    log-scales N(-4.5, 1), opacity logits N(0, 1.5), SH degree 3 (DC U[0,1],
    higher bands N(0, 0.05)); one camera on the radius-8 sphere looking at
    the origin, 50 deg, 1920x1080, 16x16 tiles.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .camera import CameraInfo, look_at_c2w

SH_C0 = 0.28209479177387814


def _raw(seed: int, stream: int, n: int) -> np.ndarray:
    bg = np.random.PCG64(np.random.SeedSequence([int(seed), int(stream)]))
    return bg.random_raw(int(n))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """float64 in [0, 1)."""
    return (_raw(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    m = (int(n) + 1) // 2
    u = uniform(seed, stream, 2 * m)
    u1 = 1.0 - u[:m]  # (0, 1]
    u2 = u[m:]
    r = np.sqrt(-2.0 * np.log(u1))
    th = 2.0 * np.pi * u2
    return np.concatenate([r * np.cos(th), r * np.sin(th)])[: int(n)]


@dataclass
class Scene:
    mean: np.ndarray         # [N,3] f32
    qvec: np.ndarray         # [N,4] f32, WXYZ
    log_scale: np.ndarray    # [N,3] f32 (svec_before_activation)
    sh: np.ndarray           # [N,3,C*C] f32
    alpha_logit: np.ndarray  # [N] f32 (alpha_before_activation)
    sh_order: int            # C = degree + 1

    @property
    def n(self) -> int:
        return int(self.mean.shape[0])


@dataclass
class View:
    c2w: np.ndarray          # [3,4] f32
    cam: CameraInfo
    tile: int = 16


@dataclass
class Workload:
    name: str
    scene: Scene
    views: list = field(default_factory=list)
    grad_weight: np.ndarray | None = None  # dL/dimage for loss = sum(image * W), [H,W,3]


def _quats(seed: int, stream: int, n: int) -> np.ndarray:
    q = normal(seed, stream, 4 * n).reshape(n, 4)
    q = q / np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def make_scene(n: int, seed: int, *, mean_dist: str, log_scale_mu: float, log_scale_sigma: float,
               alpha_sigma: float, sh_degree: int, dc_from_rgb: bool, rest_sigma: float = 0.05) -> Scene:
    if mean_dist == "uniform":
        mean = (uniform(seed, 1, 3 * n) * 2.0 - 1.0).reshape(n, 3)
    elif mean_dist == "normal2":
        mean = np.clip(normal(seed, 1, 3 * n) * 2.0, -6.0, 6.0).reshape(n, 3)
    else:
        raise ValueError(mean_dist)
    log_s = (normal(seed, 2, 3 * n) * log_scale_sigma + log_scale_mu).reshape(n, 3)
    q = _quats(seed, 3, n)
    alpha_logit = normal(seed, 4, n) * alpha_sigma
    C = sh_degree + 1
    sh = np.zeros((n, 3, C * C), dtype=np.float64)
    dc = uniform(seed, 5, 3 * n).reshape(n, 3)
    if dc_from_rgb:
        rgb = np.clip(dc, 1e-3, 1.0 - 1e-3)
        sh[:, :, 0] = np.log(rgb / (1.0 - rgb)) / SH_C0
    else:
        sh[:, :, 0] = dc
    if C > 1:
        sh[:, :, 1:] = (normal(seed, 6, n * 3 * (C * C - 1)) * rest_sigma).reshape(n, 3, C * C - 1)
    return Scene(mean.astype(np.float32), q, log_s.astype(np.float32), sh.astype(np.float32),
                 alpha_logit.astype(np.float32), C)


def sphere_direction(seed: int, stream: int, k: int) -> np.ndarray:
    v = normal(seed, stream, 3 * k).reshape(k, 3)
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def small_workload(seed: int = 0, n: int = 10_000, width: int = 256, height: int = 256) -> Workload:
    scene = make_scene(n, seed, mean_dist="uniform", log_scale_mu=-3.0, log_scale_sigma=0.5,
                       alpha_sigma=1.0, sh_degree=0, dc_from_rgb=True)
    cam = CameraInfo.from_vertical_fov(60.0, width, height)
    view = View(look_at_c2w((0.0, 0.0, -4.0)), cam, 16)
    W = uniform(seed, 7, height * width * 3).reshape(height, width, 3).astype(np.float32)
    return Workload("small", scene, [view], W)


def headline_workload(seed: int = 0, n: int = 1_000_000, width: int = 1920, height: int = 1080,
                      sh_degree: int = 3) -> Workload:
    scene = make_scene(n, seed, mean_dist="normal2", log_scale_mu=-4.5, log_scale_sigma=1.0,
                       alpha_sigma=1.5, sh_degree=sh_degree, dc_from_rgb=False)
    d = sphere_direction(seed, 8, 1)[0]
    cam = CameraInfo.from_vertical_fov(50.0, width, height)
    view = View(look_at_c2w(8.0 * d), cam, 16)
    W = uniform(seed, 7, height * width * 3).reshape(height, width, 3).astype(np.float32)
    return Workload("headline", scene, [view], W)


def batch_workload(seed: int = 0, n: int = 500_000, n_views: int = 32, radius: float = 6.0,
                   fov: float = 60.0, sizes=((800, 800), (1280, 720), (1920, 1080))) -> Workload:
    """Multi-view batching workload: Gaussians drawn as in ``small`` (means
    U[-1,1]^3, log-scales N(-3, 0.5), opacity logits N(0,1), DC from RGB
    U[0,1]) with SH degree 3 (higher bands N(0, 0.05)); n_views cameras
    uniform on the radius-6 sphere looking at the origin, image sizes cycling
    through `sizes`.  grad_weight is None: each view's dL/dimage is drawn by
    the caller."""
    scene = make_scene(n, seed, mean_dist="uniform", log_scale_mu=-3.0, log_scale_sigma=0.5,
                       alpha_sigma=1.0, sh_degree=3, dc_from_rgb=True)
    dirs = sphere_direction(seed, 10, n_views)
    views = []
    for i in range(n_views):
        w, h = sizes[i % len(sizes)]
        views.append(View(look_at_c2w(radius * dirs[i]), CameraInfo.from_vertical_fov(fov, w, h), 16))
    return Workload("batch", scene, views, None)


def custom_workload(n: int, width: int, height: int, sh_degree: int, seed: int = 0,
                    radius: float = 4.0, fov: float = 60.0, tile: int = 16,
                    log_scale_mu: float = -3.0) -> Workload:
    """Small scenes for parity tests: config-1 style Gaussians, any SH degree,
    image size and camera distance."""
    scene = make_scene(n, seed, mean_dist="uniform", log_scale_mu=log_scale_mu, log_scale_sigma=0.5,
                       alpha_sigma=1.0, sh_degree=sh_degree, dc_from_rgb=True, rest_sigma=0.3)
    d = sphere_direction(seed, 8, 1)[0]
    cam = CameraInfo.from_vertical_fov(fov, width, height)
    view = View(look_at_c2w(radius * d), cam, tile)
    W = uniform(seed, 7, height * width * 3).reshape(height, width, 3).astype(np.float32)
    return Workload(f"custom_{n}_{width}x{height}_C{sh_degree + 1}", scene, [view], W)


def diff_workload(seed: int = 0, n: int = 2000, width: int = 64, height: int = 64, sh_degree: int = 1,
                  log_scale_mu: float = -3.0, alpha_mu: float = 0.0) -> Workload:
    """Differentiation workload: Gaussians drawn as in ``small`` (means
    U[-1,1]^3, log-scales N(log_scale_mu, 0.5), opacity logits
    N(alpha_mu, 1), DC from RGB U[0,1]) with SH degree 1 (band 1 N(0, 0.3));
    camera at (0,0,-4) looking at the origin, 60 deg, 64x64, 16x16 tiles;
    loss weights W uniform in [0,1]."""
    scene = make_scene(n, seed, mean_dist="uniform", log_scale_mu=log_scale_mu, log_scale_sigma=0.5,
                       alpha_sigma=1.0, sh_degree=sh_degree, dc_from_rgb=True, rest_sigma=0.3)
    if alpha_mu:
        scene.alpha_logit = (scene.alpha_logit + np.float32(alpha_mu)).astype(np.float32)
    cam = CameraInfo.from_vertical_fov(60.0, width, height)
    view = View(look_at_c2w((0.0, 0.0, -4.0)), cam, 16)
    W = uniform(seed, 7, height * width * 3).reshape(height, width, 3).astype(np.float32)
    return Workload(f"diff_{n}_{width}x{height}_C{sh_degree + 1}", scene, [view], W)

