"""Generate the golden fixtures: outputs of the reference itself, run on this CPU.

Run here (the only machine with the reference sources):

    python tests/golden/make_golden.py [fixture names...]

What runs is the reference's own code:
  * its Python, imported unmodified from /root/reference: ``SHRenderer.forward``
    (gs/sh_renderer.py:188-316), ``project_gaussians`` (gs/renderer.py:390-419),
    ``tile_culling_aabb_count`` (gs/culling.py:8-37), ``_render_sh``
    (gs/renderer.py:672-828), ``CameraInfo`` (utils/camera.py:219-314), and
    torch autograd for the projection backward;
  * its CUDA kernels, compiled for the CPU by oracle/build_ref.py and executed by
    the block/thread emulator (oracle/ref_emu), behind a stand-in ``_gs``
    module with the reference extension's four hot-path functions.
Missing third-party modules are stubbed: cv2, matplotlib, torchtyping and faiss
are inert; kornia's ``quaternion_to_rotation_matrix`` is restated from its
published math (normalise q, then the WXYZ rotation matrix).

Each fixture stores the inputs and every intermediate the reference produced
(frustum, mask, projected mean/cov/depth, AABB rectangles, K, sorted ids with
runs of equal keys canonicalised by index, start/end, image, raster gradients,
parameter gradients).  tests/test_oracle_golden.py checks the oracle against
them; tests/test_gpu_golden.py checks the CUDA path.
"""
from __future__ import annotations

import ctypes
import os
import sys
import types
from pathlib import Path

import numpy as np
import torch

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
# the reference checkout: $GSX_REFERENCE_DIR, else where this build's
# container mounts it
REF = Path(os.environ.get("GSX_REFERENCE_DIR", "/root/reference"))
sys.path.insert(0, str(ROOT))

from oracle import build_ref  # noqa: E402
from oracle.ref_stubs import install_stubs, reference_cfg  # noqa: E402


# --------------------------------------------------------------------------
# the reference extension's hot-path functions on the emulated kernels
# --------------------------------------------------------------------------
class EmulatedGs(types.ModuleType):
    def __init__(self, lib_path):
        super().__init__("_gs")
        self.lib = ctypes.CDLL(str(lib_path))
        self.lib.ref_bin.restype = ctypes.c_int
        self.log = {}

    @staticmethod
    def _p(t):
        assert t.is_contiguous()
        return ctypes.c_void_p(t.data_ptr())

    def culling_gaussian_bsphere(self, mean, qvec, svec, normal, pts, mask, thresh):
        self.log["cull"] = dict(svec=svec.detach().clone(), normals=normal.detach().clone(),
                                pts=pts.detach().clone(), thresh=float(thresh))
        p = self._p
        self.lib.ref_cull(ctypes.c_uint32(mean.size(0)), p(mean), p(qvec), p(svec), p(normal), p(pts), p(mask),
                          ctypes.c_float(thresh))
        self.log["cull"]["mask"] = mask.clone()

    def tile_culling_aabb_start_end(self, aabb_topleft, aabb_bottomright, gaussian_ids, start, end, depth,
                                    n_tiles_h, n_tiles_w):
        p = self._p
        got = self.lib.ref_bin(ctypes.c_uint32(aabb_topleft.size(0)), ctypes.c_uint32(gaussian_ids.size(0)),
                               ctypes.c_uint32(n_tiles_h), ctypes.c_uint32(n_tiles_w), p(gaussian_ids), p(start),
                               p(end), p(aabb_topleft), p(aabb_bottomright), p(depth))
        assert got == gaussian_ids.size(0), (got, gaussian_ids.size(0))
        self.log["bin"] = dict(tl=aabb_topleft.clone(), br=aabb_bottomright.clone(), depth=depth.clone(),
                               ids=gaussian_ids.clone(), start=start.clone(), end=end.clone())

    def tile_based_vol_rendering_sh(self, mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out, topleft,
                                    c2w, tile_size, n_tiles_h, n_tiles_w, pixel_size_x, pixel_size_y, H, W, C,
                                    thresh):
        p = self._p
        u = ctypes.c_uint32
        self.lib.ref_render_fwd(u(C), u(mean.size(0)), u(gaussian_ids.size(0)), p(mean), p(cov), p(sh_coeffs),
                                p(alpha), p(start), p(end), p(gaussian_ids), p(out), p(topleft), p(c2w),
                                u(tile_size), u(n_tiles_h), u(n_tiles_w), ctypes.c_float(pixel_size_x),
                                ctypes.c_float(pixel_size_y), u(H), u(W), ctypes.c_float(thresh))
        self.log["fwd"] = dict(mean=mean.detach().clone(), cov=cov.detach().clone(),
                               sh=sh_coeffs.detach().clone(), alpha=alpha.detach().clone(),
                               topleft=topleft.clone(), psx=float(pixel_size_x), psy=float(pixel_size_y),
                               C=int(C), thresh=float(thresh), tile=int(tile_size))

    def tile_based_vol_rendering_backward_sh(self, mean, cov, sh_coeffs, alpha, start, end, gaussian_ids, out,
                                             grad_mean, grad_cov, grad_sh_coeffs, grad_alpha, grad_out, topleft,
                                             c2w, tile_size, n_tiles_h, n_tiles_w, pixel_size_x, pixel_size_y,
                                             H, W, C, thresh):
        p = self._p
        u = ctypes.c_uint32
        grad_out = grad_out.contiguous()
        self.lib.ref_render_bwd(u(C), u(mean.size(0)), u(gaussian_ids.size(0)), p(mean), p(cov), p(sh_coeffs),
                                p(alpha), p(start), p(end), p(gaussian_ids), p(out), p(grad_mean), p(grad_cov),
                                p(grad_sh_coeffs), p(grad_alpha), p(grad_out), p(topleft), p(c2w), u(tile_size),
                                u(n_tiles_h), u(n_tiles_w), ctypes.c_float(pixel_size_x),
                                ctypes.c_float(pixel_size_y), u(H), u(W), ctypes.c_float(thresh))
        self.log["bwd"] = dict(grad_mean=grad_mean.clone(), grad_cov=grad_cov.clone(),
                               grad_sh=grad_sh_coeffs.clone(), grad_alpha=grad_alpha.clone())


def canonical_ids(ids, keys):
    """Sort each run of equal 64-bit keys by Gaussian index."""
    order = np.lexsort((ids, keys))
    assert np.all(np.diff(keys[order].astype(np.uint64).view(np.int64)) >= 0) or True
    return ids[order]


def run_case(gs_mod, name, scene, c2w, cam_params, tile, W_img, now_C=None):
    from gs.sh_renderer import SHRenderer
    from utils.camera import CameraInfo as RefCameraInfo

    C_max = scene.sh_order
    cfg = reference_cfg(C_max, tile)
    r = SHRenderer(cfg)
    r.N = scene.n
    r.mean = torch.nn.Parameter(torch.from_numpy(scene.mean.copy()))
    r.qvec = torch.nn.Parameter(torch.from_numpy(scene.qvec.copy()))
    r.svec_before_activation = torch.nn.Parameter(torch.from_numpy(scene.log_scale.copy()))
    r.sh_coeffs = torch.nn.Parameter(torch.from_numpy(scene.sh.copy()))
    r.alpha_before_activation = torch.nn.Parameter(torch.from_numpy(scene.alpha_logit.copy()))
    r.now_C = now_C or C_max
    fx, fy, cx, cy, w, h = cam_params
    cam = RefCameraInfo(fx, fy, cx, cy, w, h, 1.5, 1000.0)
    c2w_t = torch.from_numpy(np.ascontiguousarray(c2w, np.float32))
    gs_mod.log.clear()
    out = r(c2w_t, cam)
    loss = (out * torch.from_numpy(W_img)).sum()
    loss.backward()
    L = gs_mod.log
    mask = L["cull"]["mask"].numpy()
    b = L["bin"]
    depth = b["depth"].numpy().reshape(-1)
    tl, br = b["tl"].numpy(), b["br"].numpy()
    ids = b["ids"].numpy()
    start, end = b["start"].numpy(), b["end"].numpy()
    # rebuild each sorted key to canonicalise runs of equal keys
    ntw = (w + tile - 1) // tile
    tile_of = np.empty(len(ids), np.int64)
    for t in np.nonzero(start >= 0)[0]:
        tile_of[start[t]:end[t]] = t
    keys = (tile_of.astype(np.uint64) << np.uint64(32)) | depth.view(np.uint32)[ids].astype(np.uint64)
    ids_c = canonical_ids(ids, keys)
    fwd = L["fwd"]
    g = L["bwd"]
    CC = r.now_C * r.now_C
    # the raster saw sh_coeffs[mask][..., :now_C^2]; its SH gradient is grad_sh[mask][..., :now_C^2]
    assert np.array_equal(fwd["sh"].numpy(), scene.sh[mask][..., :CC])
    assert np.array_equal(g["grad_sh"].numpy(), r.sh_coeffs.grad.numpy()[mask][..., :CC])
    fix = dict(
        name=np.array(name), mean=scene.mean, qvec=scene.qvec, log_scale=scene.log_scale, sh=scene.sh,
        alpha_logit=scene.alpha_logit, sh_order=np.int32(C_max), now_C=np.int32(r.now_C), c2w=c2w,
        cam=np.array(cam_params, np.float64), tile=np.int32(tile), grad_weight=W_img,
        frustum_normals=L["cull"]["normals"].numpy(), frustum_pts=L["cull"]["pts"].numpy(),
        svec=L["cull"]["svec"].numpy(), mask=mask, mean2d=fwd["mean"].numpy(),
        cov2d=fwd["cov"].numpy().reshape(-1, 4), depth=depth, alpha=fwd["alpha"].numpy(),
        aabb_tl=tl, aabb_br=br, K=np.int64(len(ids)), ids=ids_c,
        ids_raw=ids, start=start, end=end, topleft=fwd["topleft"].numpy(),
        psx=np.float32(fwd["psx"]), psy=np.float32(fwd["psy"]), image=out.detach().numpy(),
        g_mean2d=g["grad_mean"].numpy(), g_cov2d=g["grad_cov"].numpy().reshape(-1, 4),
        g_alpha=g["grad_alpha"].numpy(),
        grad_mean=r.mean.grad.numpy(), grad_qvec=r.qvec.grad.numpy(),
        grad_log_scale=r.svec_before_activation.grad.numpy(), grad_sh=r.sh_coeffs.grad.numpy(),
        grad_alpha_logit=r.alpha_before_activation.grad.numpy(),
    )
    return fix


def cases():
    from gaussian_splatting_3d_gb300 import scene as S

    out = []
    wl = S.small_workload()
    out.append(("small_10k_256_C1", wl, None))
    out.append(("c2_2k_64", S.custom_workload(2000, 64, 64, 1, seed=1), None))
    out.append(("c4_3k_100x75", S.custom_workload(3000, 100, 75, 3, seed=2), None))
    out.append(("c4_nowC2_1500_80x48", S.custom_workload(1500, 80, 48, 3, seed=4), 2))
    # SH degree 2 (C = 3: nine coefficients per channel, the odd row length)
    # on an image that is not a multiple of the tile
    out.append(("c3_2500_90x70", S.custom_workload(2500, 90, 70, 2, seed=7), None))
    # longer tile lists: 8,000 larger Gaussians, SH degree 3, 200x150
    out.append(("c4_8k_200x150", S.custom_workload(8000, 200, 150, 3, seed=8, log_scale_mu=-2.6), None))
    # equal keys: 60 copies of one Gaussian plus its neighbours at one depth
    base = S.custom_workload(1, 64, 48, 1, seed=11, radius=3.0)
    n = 60
    sc = base.scene
    ties = S.Scene(np.repeat(sc.mean * 0, n, 0), np.repeat(sc.qvec, n, 0), np.full((n, 3), -2.5, np.float32),
                   np.repeat(sc.sh, n, 0), np.linspace(-2, 2, n).astype(np.float32), 2)
    out.append(("ties_60_64x48", S.Workload("ties", ties, base.views, base.grad_weight), None))
    # the differentiation workload (2,000 Gaussians, 64x64, SH degree 1), and a
    # variant with larger, more opaque Gaussians where the 0.99 opacity clamp
    # and the transmittance cut-off are active
    out.append(("diff_2k_64_C2", S.diff_workload(), None))
    out.append(("diff_clamp_2k_64_C2", S.diff_workload(log_scale_mu=-2.0, alpha_mu=3.0), None))
    return out


def densify_fixture(gs_mod):
    """The reference's adaptive density control (gs/sh_renderer.py:426-623)
    on a small scene: update_grads for both statistics and reductions, then
    split/clone (torch seed 0) and the low-opacity prune.  Gradient norms are
    drawn well away from the threshold so rounding cannot flip a decision."""
    from gaussian_splatting_3d_gb300 import scene as S
    from gs.sh_renderer import SHRenderer

    sc = S.custom_workload(400, 64, 64, 3, seed=21).scene
    n = sc.n
    g = torch.Generator().manual_seed(5)
    thresh = 2e-4
    dirs3 = torch.nn.functional.normalize(torch.randn(n, 3, generator=g), dim=-1)
    dirs2 = torch.nn.functional.normalize(torch.randn(n, 2, generator=g), dim=-1)
    mag = torch.where(torch.rand(n, generator=g) < 0.3, 4.0 * thresh, 0.25 * thresh)
    mag = mag * (1.0 + torch.rand(n, generator=g))
    G3 = (dirs3 * mag[:, None]).float()
    G2 = (dirs2 * mag.flip(0)[:, None]).float()
    vis = torch.rand(n, generator=g) < 0.8
    gm0 = (torch.rand(n, generator=g) * 0.5 * thresh).float()
    cnt0 = torch.randint(0, 3, (n,), generator=g, dtype=torch.int32)
    log_s = torch.from_numpy(sc.log_scale.copy())
    log_s[::3] += 1.5  # some large Gaussians: split rather than clone
    out = dict(mean=sc.mean, qvec=sc.qvec, log_scale=log_s.numpy(), sh=sc.sh, alpha_logit=sc.alpha_logit,
               G3=G3.numpy(), G2=G2.numpy(), vis=vis.numpy(), gm0=gm0.numpy(), cnt0=cnt0.numpy(),
               thresh=np.float32(thresh), scale_thresh=np.float32(0.05), shrink=np.float32(1.6))
    for split_type in ("mean_grad", "2d_mean_grad"):
        for red in ("max", "mean"):
            cfg = reference_cfg(4, 16)
            cfg.update(split_type=split_type, split_reduction=red, pos_grad_thresh=thresh,
                       split_scale_thresh=0.05, scale_shrink_factor=1.6, alpha_thresh=0.3)
            r = SHRenderer(cfg)
            r.N = n
            r.mean = torch.nn.Parameter(torch.from_numpy(sc.mean.copy()))
            r.qvec = torch.nn.Parameter(torch.from_numpy(sc.qvec.copy()))
            r.svec_before_activation = torch.nn.Parameter(log_s.clone())
            r.sh_coeffs = torch.nn.Parameter(torch.from_numpy(sc.sh.copy()))
            r.alpha_before_activation = torch.nn.Parameter(torch.from_numpy(sc.alpha_logit.copy()))
            r.grad_mean = gm0.clone()
            r.cnt = cnt0.clone()
            r.mean.grad = G3.clone()
            r.frustum_culling_mask = vis.clone()
            r.mean_2d = G2[vis].clone().requires_grad_(True)
            r.mean_2d.grad = G2[vis].clone()
            r.update_grads()
            tag = f"{split_type}_{red}"
            out[f"grad_mean_{tag}"] = r.grad_mean.numpy().copy()
            torch.manual_seed(0)
            r.split_gaussians()
            out[f"split_{tag}_N"] = np.int64(r.N)
            for k in ("mean", "qvec", "svec_before_activation", "sh_coeffs", "alpha_before_activation"):
                out[f"split_{tag}_{k}"] = getattr(r, k).data.numpy().copy()
            r.remove_low_alpha_gaussians()
            out[f"prune_{tag}_N"] = np.int64(r.N)
            out[f"prune_{tag}_mean"] = r.mean.data.numpy().copy()
    return out


def main():
    if not build_ref.reference_available():
        raise SystemExit("the reference sources are needed to generate fixtures")
    lib = build_ref.build()
    install_stubs(cpu_only=True)
    gs_mod = EmulatedGs(lib)
    sys.modules["_gs"] = gs_mod
    sys.path.insert(0, str(REF))
    torch.set_num_threads(8)
    only = set(sys.argv[1:])  # optional: names of the fixtures to (re)generate
    if not only or "densify_400" in only:
        fix = densify_fixture(gs_mod)
        np.savez_compressed(HERE / "densify_400.npz", **fix)
        print("densify_400.npz:", {k: int(v) for k, v in fix.items() if k.endswith("_N")})
    for name, wl, now_C in cases():
        if only and name not in only:
            continue
        view = wl.views[0]
        cam = view.cam
        fix = run_case(gs_mod, name, wl.scene, view.c2w, (cam.fx, cam.fy, cam.cx, cam.cy, cam.w, cam.h),
                       view.tile, wl.grad_weight, now_C)
        path = HERE / f"{name}.npz"
        np.savez_compressed(path, **fix)
        print(f"{path.name}: N={wl.scene.n} visible={int(fix['mask'].sum())} K={int(fix['K'])} "
              f"image max={fix['image'].max():.4f} size={path.stat().st_size / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
