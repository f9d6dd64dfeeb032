"""FP64 dense restatement of the SH Gaussian-splatting forward, differentiable
with torch autograd.

TEST INFRASTRUCTURE ONLY: the checker for the gradient modes of the
hand-written backward (finite differences and autograd in float64).  Only the
tests import it; the product never does.

The function restated is the renderer's forward exactly as the C oracle
(oracle/gsx_oracle.c) and the kernels compute it, with every discrete choice
taken the same way:
  * activations scale = exp(log_scale), opacity = sigmoid(logit)
    (utils/activations.py:13-19);
  * bounding-sphere frustum culling with radius max(scale) * frustum radius
    (gs/src/include/culling.h:11-20);
  * p = W (mean - t) with W the transposed rotation of c2w, mean2d = p_xy / z,
    cov2d = A Sigma A^T with A = J(p) W and Sigma = M M^T, M = R(q) diag(scale),
    R from the normalised WXYZ quaternion (gs/renderer.py:365-419,
    utils/transforms.py:31-45);
  * the AABB tile rectangle of half-widths sqrt(tile_radius * cov_xx),
    sqrt(tile_radius * cov_yy), truncated toward zero in pixels, clamped and
    divided by the tile size (gs/culling.py:8-37, utils/camera.py:290-303);
  * per tile, the Gaussians whose rectangle covers it in increasing depth;
    per pixel the SH basis of the ray read from the flat c2w array as rows
    (vol_render_sh.h:208-217), colour sigmoid(sh . Y), G = exp(-radial / 2)
    with radial < 0 -> 1000, alpha = min(opacity, 0.99) G, skipped below
    1/255, front-to-back with the transmittance test T < T_thresh before each
    Gaussian (vol_render_sh.h:120-168).

Gradient modes (what autograd differentiates):
  * ``exact``: the true derivative of that function;
  * ``parity``: the reference's gradient -- depth detached in mean2d
    (gs/renderer.py:408-417), J built without gradient (gs/renderer.py:365-377),
    the opacity clamp passed straight through (vol_render_sh.h:346);
  * ``depth``: parity with depth_detach=False (gs/sh_renderer.py:144).

Camera constants (c2w, fx, fy, cx, cy, topleft, pixel size) are the float32
values the kernels receive, widened to float64.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

F64 = torch.float64
MIN_ALPHA = float(np.float32(1.0 / 255.0))
SH_C = [0.28209479177387814, 0.48860251190291987, 1.0925484305920792, 0.94617469575755997,
        0.31539156525251999, 0.54627421529603959, 0.59004358992664352, 2.8906114426405538,
        0.45704579946446572, 0.3731763325901154, 1.4453057213202769]


@dataclass
class Cam64:
    c2w: torch.Tensor        # [12] float64 (float32 values)
    fx: float
    fy: float
    cx: float
    cy: float
    w: int
    h: int
    normals: torch.Tensor    # [6,3]
    pts: torch.Tensor        # [6,3]
    topleft: tuple
    psx: float
    psy: float

    @classmethod
    def from_view(cls, c2w, cam, device="cpu") -> "Cam64":
        from gaussian_splatting_3d_gb300.camera import frustum_np

        c2w32 = np.ascontiguousarray(c2w, dtype=np.float32).reshape(3, 4)
        normals, pts = frustum_np(c2w32, cam)
        tl = np.array(cam.topleft(), np.float32)
        f = lambda v: float(np.float32(v))  # noqa: E731
        return cls(torch.tensor(c2w32.reshape(-1), dtype=F64, device=device), f(cam.fx), f(cam.fy), f(cam.cx),
                   f(cam.cy), int(cam.w), int(cam.h), torch.tensor(normals, dtype=F64, device=device),
                   torch.tensor(pts, dtype=F64, device=device), (float(tl[0]), float(tl[1])),
                   float(np.float32(1.0 / cam.fx)), float(np.float32(1.0 / cam.fy)))


@dataclass
class Settings64:
    tile_w: int = 16
    tile_h: int = 16
    frustum_radius: float = 1.0
    tile_radius: float = 6.0
    T_thresh: float = float(np.float32(0.01))


def quat_rot(q: torch.Tensor) -> torch.Tensor:
    """[..., 4] WXYZ -> [..., 3, 3], quaternion normalised first."""
    q = q / q.norm(dim=-1, keepdim=True).clamp_min(1e-12)
    w, x, y, z = q.unbind(-1)
    return torch.stack([
        1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
        2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
        2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1).reshape(q.shape[:-1] + (3, 3))


def project(mean, qvec, log_scale, alpha_logit, cam: Cam64, st: Settings64, mode: str):
    """Per-Gaussian projection (any leading batch shape [..., N]).  Returns
    mean2d [...,2], cov [...,4], depth [...], opacity after the clamp [...],
    rect [...,4] (int64, no grad) and keep [...] (bool)."""
    s = torch.exp(log_scale)
    o = torch.sigmoid(alpha_logit)
    with torch.no_grad():
        r = s.max(dim=-1).values * st.frustum_radius
        d = ((mean.unsqueeze(-2) - cam.pts) * cam.normals).sum(-1)  # [..., N, 6]
        keep = (d > -r.unsqueeze(-1)).all(-1)
    R = cam.c2w.reshape(3, 4)[:, :3]
    t = cam.c2w.reshape(3, 4)[:, 3]
    p = (mean - t) @ R  # p = W (mean - t), W = R^T
    Rq = quat_rot(qvec)
    M = Rq * s.unsqueeze(-2)
    Sig = M @ M.transpose(-1, -2)
    if mode not in ("parity", "depth", "exact"):
        raise ValueError(mode)
    pj = p if mode == "exact" else p.detach()  # J without gradient unless exact
    x, y, z = pj.unbind(-1)
    zero = torch.zeros_like(z)
    J = torch.stack([1 / z, zero, -x / (z * z), zero, 1 / z, -y / (z * z)], -1).reshape(z.shape + (2, 3))
    A = J @ R.t()
    cov = (A @ Sig @ A.transpose(-1, -2)).reshape(z.shape + (4,))
    zd = p[..., 2].detach() if mode == "parity" else p[..., 2]
    mean2d = p[..., :2] / zd.unsqueeze(-1)
    if mode != "exact":
        opac = o - (o - 0.99).clamp_min(0.0).detach()  # value min(o, 0.99), gradient 1
    else:
        opac = o.clamp_max(0.99)
    with torch.no_grad():
        ax = torch.sqrt(st.tile_radius * cov[..., 0])
        ay = torch.sqrt(st.tile_radius * cov[..., 3])
        mx, my = mean2d[..., 0], mean2d[..., 1]

        def tile(v, f, c, size, limit):
            pix = torch.nan_to_num(torch.trunc(v * f + c), nan=0.0).clamp(-2.0 ** 31, 2.0 ** 31 - 1)
            return torch.div(pix.to(torch.int64).clamp(0, limit - 1), size, rounding_mode="floor")

        rect = torch.stack([tile(mx - ax, cam.fx, cam.cx, st.tile_w, cam.w),
                            tile(my - ay, cam.fy, cam.cy, st.tile_h, cam.h),
                            tile(mx + ax, cam.fx, cam.cx, st.tile_w, cam.w),
                            tile(my + ay, cam.fy, cam.cy, st.tile_h, cam.h)], -1)
    return dict(mean2d=mean2d, cov=cov, depth=p[..., 2], opac=opac, rect=rect, keep=keep)


def sh_basis(cam: Cam64, px, py, C: int, sh_dir: str = "reference"):
    """Per-pixel SH basis; "reference": the direction from the flat c2w read
    with a row stride of 3 (vol_render_sh.h:48-65); "ray": R (x, y, 1)."""
    c = cam.c2w
    s = 3 if sh_dir == "reference" else 4
    d = torch.stack([c[s * r] * px + c[s * r + 1] * py + c[s * r + 2] for r in range(3)], -1)
    return sh_basis_dir(d / d.norm(dim=-1, keepdim=True), C)


def gaussian_colors(mean, sh, cam: Cam64, C: int):
    """Per-Gaussian colours of the opt-in mode: sigmoid(sh . Y(dir)) with dir
    the unit vector from the camera centre (c2w[:, 3]) to the mean; [..., N, 3]."""
    d = mean - cam.c2w.reshape(3, 4)[:, 3]
    Y = sh_basis_dir(d / d.norm(dim=-1, keepdim=True), C)           # [..., N, C*C]
    return torch.sigmoid((sh[..., :C * C] * Y.unsqueeze(-2)).sum(-1))


def sh_basis_dir(d, C: int):
    """Real SH basis (shencoder.h:13-58) at unit directions d [..., 3]."""
    x, y, z = d.unbind(-1)
    Y = [torch.full_like(x, SH_C[0])]
    if C > 1:
        Y += [-SH_C[1] * y, SH_C[1] * z, -SH_C[1] * x]
    if C > 2:
        Y += [SH_C[2] * x * y, -SH_C[2] * y * z, SH_C[3] * z * z - SH_C[4], -SH_C[2] * x * z,
              SH_C[5] * x * x - SH_C[5] * y * y]
    if C > 3:
        Y += [SH_C[6] * y * (y * y - 3 * x * x), SH_C[7] * x * y * z, SH_C[8] * y * (1 - 5 * z * z),
              SH_C[9] * z * (5 * z * z - 3), SH_C[8] * x * (1 - 5 * z * z), SH_C[10] * z * (x * x - y * y),
              SH_C[6] * x * (3 * y * y - x * x)]
    return torch.stack(Y, -1)


def tile_pixels(cam: Cam64, st: Settings64, tx: int, ty: int, device):
    gx = torch.arange(tx * st.tile_w, min((tx + 1) * st.tile_w, cam.w), device=device)
    gy = torch.arange(ty * st.tile_h, min((ty + 1) * st.tile_h, cam.h), device=device)
    GY, GX = torch.meshgrid(gy, gx, indexing="ij")
    GX, GY = GX.reshape(-1), GY.reshape(-1)
    px = cam.topleft[0] + GX.to(F64) * cam.psx
    py = cam.topleft[1] + GY.to(F64) * cam.psy
    return GX, GY, px, py


def composite(px, py, Y, mean2d, cov, opac, sh, member, T_thresh, extras: bool = False, z=None, rgb=None):
    """Pixels [P] x depth-ordered Gaussians [..., M] -> colours [..., P, 3]
    (with extras: also the final transmittance [..., P] and the depth sum
    sum T a G z [..., P]).  member [..., M] masks Gaussians that are not on
    this tile's list.  rgb [..., M, 3]: per-Gaussian colours instead of the
    per-pixel SH colour."""
    dx = px.unsqueeze(-1) - mean2d[..., None, :, 0]
    dy = py.unsqueeze(-1) - mean2d[..., None, :, 1]
    c0, c1, c2, c3 = (cov[..., None, :, k] for k in range(4))
    det = c0 * c3 - c1 * c2
    tmpx = dx * c3 - dy * c2
    tmpy = -dx * c1 + dy * c0
    radial = (tmpx * dx + tmpy * dy) / det
    radial = torch.where(radial < 0, torch.full_like(radial, 1000.0), radial)
    G = torch.exp(-0.5 * radial)
    aG = opac[..., None, :] * G
    valid = (aG >= MIN_ALPHA) & member[..., None, :]
    eff = torch.where(valid, aG, torch.zeros_like(aG))
    Tin = torch.cumprod(1.0 - eff, dim=-1)
    T = torch.cat([torch.ones_like(Tin[..., :1]), Tin[..., :-1]], -1)
    inc = valid & (T >= T_thresh)
    wgt = torch.where(inc, T * eff, torch.zeros_like(eff))             # [..., P, M]
    if rgb is not None:
        col = rgb.unsqueeze(-3)                                         # [..., 1, M, 3]
    else:
        col = torch.sigmoid(torch.einsum("...mck,pk->...pmc", sh, Y))  # [..., P, M, 3]
    rgb = (wgt.unsqueeze(-1) * col).sum(-2)
    if not extras:
        return rgb
    T_final = torch.where(inc, 1.0 - eff, torch.ones_like(eff)).prod(-1)
    dsum = (wgt * z[..., None, :]).sum(-1) if z is not None else None
    return rgb, T_final, dsum


def render(mean, qvec, log_scale, sh, alpha_logit, cam: Cam64, st: Settings64, C: int, mode: str = "exact",
           bg=None, maps: bool = False, sh_mode: str = "pixel", sh_dir: str = "reference"):
    """Full image [H, W, 3] (float64, differentiable); bg: background RGB
    composited behind (out += T_final bg); maps: also return the alpha map
    (1 - T_final) and the depth map (sum T a G z), [H, W] each; sh_mode
    "gaussian": one colour per Gaussian (gaussian_colors) instead of the
    per-pixel SH colour."""
    dev = mean.device
    pr = project(mean, qvec, log_scale, alpha_logit, cam, st, mode)
    rgb_all = gaussian_colors(mean, sh, cam, C) if sh_mode == "gaussian" else None
    img = torch.zeros((cam.h, cam.w, 3), dtype=F64, device=dev)
    Tmap = torch.ones((cam.h, cam.w), dtype=F64, device=dev)
    dmap = torch.zeros((cam.h, cam.w), dtype=F64, device=dev)
    ntw = (cam.w + st.tile_w - 1) // st.tile_w
    nth = (cam.h + st.tile_h - 1) // st.tile_h
    rect, keep = pr["rect"], pr["keep"]
    shc = sh[..., :C * C]
    for ty in range(nth):
        for tx in range(ntw):
            m = keep & (rect[:, 0] <= tx) & (rect[:, 2] >= tx) & (rect[:, 1] <= ty) & (rect[:, 3] >= ty)
            idx = torch.nonzero(m).reshape(-1)
            if idx.numel() == 0:
                continue
            idx = idx[torch.argsort(pr["depth"].detach()[idx], stable=True)]
            GX, GY, px, py = tile_pixels(cam, st, tx, ty, dev)
            Y = sh_basis(cam, px, py, C, sh_dir)
            c, Tf, ds = composite(px, py, Y, pr["mean2d"][idx], pr["cov"][idx], pr["opac"][idx], shc[idx],
                                  torch.ones(idx.numel(), dtype=torch.bool, device=dev), st.T_thresh,
                                  extras=True, z=pr["depth"][idx],
                                  rgb=rgb_all[idx] if rgb_all is not None else None)
            img = img.index_put((GY, GX), c)
            Tmap = Tmap.index_put((GY, GX), Tf)
            dmap = dmap.index_put((GY, GX), ds)
    if bg is not None:
        img = img + Tmap[..., None] * torch.as_tensor(bg, dtype=F64, device=dev)
    return (img, 1.0 - Tmap, dmap) if maps else img


def param_grads(params64, W, cam: Cam64, st: Settings64, C: int, mode: str, bg=None, sh_mode: str = "pixel",
                sh_dir: str = "reference"):
    """Autograd gradients of sum(W * image) in float64: dict of 5 tensors."""
    ps = [p.detach().clone().requires_grad_(True) for p in params64]
    img = render(*ps, cam, st, C, mode, bg=bg, sh_mode=sh_mode, sh_dir=sh_dir)
    (img * W).sum().backward()
    return dict(zip(["mean", "qvec", "log_scale", "sh", "alpha_logit"], [p.grad for p in ps])), img.detach()


def fd_gaussian(params64, W, cam: Cam64, st: Settings64, C: int, j: int, h: float = 1e-4):
    """Central differences of sum(W * image) over every parameter of Gaussian j
    (mean 3, qvec 4, log_scale 3, sh 3*C*C, alpha_logit 1), at steps h and
    h/2.  All perturbed copies of Gaussian j are evaluated in one batch over
    the tiles that any of them (or the unperturbed one) covers; the other
    Gaussians keep their projection and depth order.  Returns (fd_h, fd_h2),
    each [n_params] float64, in the order above."""
    mean, qvec, log_scale, sh, alpha_logit = params64
    dev = mean.device
    with torch.no_grad():
        theta = torch.cat([mean[j], qvec[j], log_scale[j], sh[j, :, :C * C].reshape(-1), alpha_logit[j:j + 1]])
        K = theta.numel()
        steps = torch.tensor([h, -h, h / 2, -h / 2], dtype=F64, device=dev)
        D = (torch.eye(K, dtype=F64, device=dev).unsqueeze(0) * steps.view(4, 1, 1)).reshape(4 * K, K)
        th = torch.cat([theta.unsqueeze(0), theta.unsqueeze(0) + D])   # [B = 1 + 4K, K]
        B = th.shape[0]
        pj = project(th[:, 0:3], th[:, 3:7], th[:, 7:10], th[:, -1], cam, st, "exact")
        shj = th[:, 10:10 + 3 * C * C].reshape(B, 3, C * C)
        base = project(mean, qvec, log_scale, alpha_logit, cam, st, "exact")
        rect, keep = base["rect"], base["keep"].clone()
        keep[j] = False
        rj, kj = pj["rect"], pj["keep"]
        total = torch.zeros(B, dtype=F64, device=dev)
        if not bool(kj.any()):
            z = torch.zeros(K, dtype=F64, device=dev)
            return z, z.clone()
        tiles = set()
        for b in torch.nonzero(kj).reshape(-1).tolist():
            x0, y0, x1, y1 = rj[b].tolist()
            tiles.update((tx, ty) for ty in range(y0, y1 + 1) for tx in range(x0, x1 + 1))
        shc = sh[..., :C * C]
        for tx, ty in sorted(tiles):
            m = keep & (rect[:, 0] <= tx) & (rect[:, 2] >= tx) & (rect[:, 1] <= ty) & (rect[:, 3] >= ty)
            idx = torch.nonzero(m).reshape(-1)
            idx = idx[torch.argsort(base["depth"][idx], stable=True)]
            pos = int((base["depth"][idx] < base["depth"][j]).sum())  # j's place in the depth order
            M = idx.numel() + 1

            def spliced(others, mine):
                o = others.unsqueeze(0).expand((B,) + others.shape)
                return torch.cat([o[:, :pos], mine.unsqueeze(1), o[:, pos:]], 1)

            mean2d = spliced(base["mean2d"][idx], pj["mean2d"])
            cov = spliced(base["cov"][idx], pj["cov"])
            opac = spliced(base["opac"][idx], pj["opac"])
            shs = spliced(shc[idx], shj)
            member = torch.ones((B, M), dtype=torch.bool, device=dev)
            member[:, pos] = kj & (rj[:, 0] <= tx) & (rj[:, 2] >= tx) & (rj[:, 1] <= ty) & (rj[:, 3] >= ty)
            GX, GY, px, py = tile_pixels(cam, st, tx, ty, dev)
            Y = sh_basis(cam, px, py, C)
            col = composite(px, py, Y, mean2d, cov, opac, shs, member, st.T_thresh)   # [B, P, 3]
            total += (col * W[GY, GX].unsqueeze(0)).sum((1, 2))
        L = total[1:].reshape(4, K)
        return (L[0] - L[1]) / (2 * h), (L[2] - L[3]) / h


def gaussian_param_rows(grads: dict, j: int, C: int) -> torch.Tensor:
    """Gradient entries of Gaussian j in fd_gaussian's order."""
    return torch.cat([grads["mean"][j].double(), grads["qvec"][j].double(), grads["log_scale"][j].double(),
                      grads["sh"][j, :, :C * C].reshape(-1).double(), grads["alpha_logit"][j:j + 1].double()])


def to64(scene, device="cpu"):
    return [torch.tensor(np.asarray(a), dtype=F64, device=device) for a in
            (scene.mean, scene.qvec, scene.log_scale, scene.sh, scene.alpha_logit)]
