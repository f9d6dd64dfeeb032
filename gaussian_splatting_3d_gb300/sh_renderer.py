"""``SHRenderer`` with the reference's model surface (gs/sh_renderer.py:44-324,
663-729) on the fused sm_103a path.

Same parameter tensors and names (``mean``, ``qvec``, ``svec_before_activation``,
``sh_coeffs``, ``alpha_before_activation``), same activations (exp scales,
sigmoid opacity), same SH warm-up counter ``now_C``, same checkpoint format
(``save`` / ``load``) and ``forward(c2w, camera_info) -> [H, W, 3]``.  The
forward is one fused projection + binning + raster; ``loss.backward()`` runs
the raster backward and the projection backward and fills all five ``.grad``
tensors.  Adaptive density control follows the reference's policy
(gs/sh_renderer.py:216-221, 426-660): visit counts and the gradient
statistic are updated by native kernels (csrc/densify.cu), split / clone
rewrites the parameter arrays natively, pruning and the opacity reset are
tensor masks as in the reference.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from .camera import CameraInfo
from .checkpoint import PARAM_KEYS, load_state, save_state
from . import _lib
from ._torch import ptr, stream_handle
from .renderer import RasterSettings, rasterize

SH_C0 = 0.28209479177387814


class SHRenderer(torch.nn.Module):
    def __init__(self, cfg=None, pts=None, rgb=None, sh_order: int = 4, device="cuda"):
        super().__init__()
        get = (lambda k, d: cfg.get(k, d)) if cfg is not None else (lambda k, d: d)
        self.cfg = cfg
        self.device = torch.device(get("device", device))
        self.max_C = int(get("sh_order", sh_order))
        self.now_C = 1
        self.settings = RasterSettings(
            tile_w=int(get("tile_size", 16)), tile_h=int(get("tile_size", 16)),
            frustum_culling_radius=float(get("frustum_culling_radius", 1.0)),
            tile_culling_radius=float(get("tile_culling_radius", 6.0)),
            T_thresh=float(get("T_thresh", 0.01)),
            depth_detach=bool(get("depth_detach", True)),
            exact_grad=bool(get("exact_grad", False)),
            # gs/sh_renderer.py:146-149: bg / bg_rgb (default white when enabled)
            bg=tuple(float(v) for v in get("bg_rgb", [1.0, 1.0, 1.0])) if get("bg", False) else None)
        # adaptive density control (conf/garden_sh.yaml keys, gs/sh_renderer.py:104-151)
        self.warm_up = int(get("warm_up", 1000))
        self.adaptive_control_iteration = int(get("adaptive_control_iteration", 800))
        self.pos_grad_thresh = float(get("pos_grad_thresh", 0.0002))
        self.split_scale_thresh = float(get("split_scale_thresh", 0.02))
        self.scale_shrink_factor = float(get("scale_shrink_factor", 1.6))
        self.alpha_reset_period = int(get("alpha_reset_period", 100000000))
        self.remove_low_alpha_period = int(get("remove_low_alpha_period", 10000000))
        self.alpha_reset_val = float(get("alpha_reset_val", 0.1))
        self.alpha_thresh = float(get("alpha_thresh", 0.05))
        self.split_type = str(get("split_type", "mean_grad"))
        self.split_reduction = str(get("split_reduction", "max"))
        self.sh_upgrades = list(get("sh_upgrades", []))
        self.split_seed = 0
        self.N_changed = False
        self._aux = None
        if pts is not None and rgb is not None:
            self.initialize(pts, rgb, float(get("svec_init", 0.02)), float(get("alpha_init", 0.5)))

    def initialize(self, pts, rgb, svec_init=0.02, alpha_init=0.5):
        """Fixed-scale initialisation (gs/sh_renderer.py:79-102, "fixed" method):
        DC colour = logit(rgb) / Y00, identity rotation."""
        n = pts.shape[0]
        dev = self.device
        self.N = n
        self.mean = torch.nn.Parameter(pts.to(dev, torch.float32).contiguous())
        q = torch.zeros((n, 4), device=dev)
        q[:, 0] = 1.0
        self.qvec = torch.nn.Parameter(q)
        sh = torch.zeros((n, 3, self.max_C * self.max_C), device=dev)
        sh[:, :, 0] = torch.logit(rgb.to(dev, torch.float32)) / SH_C0
        self.sh_coeffs = torch.nn.Parameter(sh)
        self.svec_before_activation = torch.nn.Parameter(
            torch.full((n, 3), float(torch.log(torch.tensor(svec_init))), device=dev))
        self.alpha_before_activation = torch.nn.Parameter(
            torch.full((n,), float(torch.logit(torch.tensor(alpha_init))), device=dev))

    @property
    def svec(self):
        return torch.exp(self.svec_before_activation)

    @property
    def alpha(self):
        return torch.sigmoid(self.alpha_before_activation)

    def forward(self, c2w, camera_info: CameraInfo):
        st = RasterSettings(**{**self.settings.__dict__, "sh_order": self.now_C})
        aux = {} if self.training else None
        img = rasterize(self.mean, self.qvec, self.svec_before_activation, self.sh_coeffs,
                        self.alpha_before_activation, c2w, camera_info, st, aux)
        if aux is not None:  # gs/sh_renderer.py:215-221
            self._ensure_stats()
            _lib.call("gsx_densify_count_visible", self.N, ptr(aux["counts"]), ptr(self.cnt),
                      stream_handle(self.device))
            self.frustum_culling_mask = aux["counts"] > 0
            self._aux = aux
        return img

    # ------------------------------------------------------ density control
    def _ensure_stats(self):
        if getattr(self, "grad_mean", None) is None or self.grad_mean.shape[0] != self.N:
            self.grad_mean = torch.zeros(self.N, dtype=torch.float32, device=self.device)
            self.cnt = torch.zeros(self.N, dtype=torch.int32, device=self.device)

    @property
    def mean_2d_grad(self):
        """dL/dmean2d of the last backward ([N, 2], zero for culled Gaussians):
        the gradient the reference reads from mean_2d.grad."""
        return None if self._aux is None else self._aux.get("mean2d_grad")

    def update_grads(self):
        """gs/sh_renderer.py:602-623: accumulate |dL/dmean| ("mean_grad") or
        |dL/dmean2d| of the visible Gaussians ("2d_mean_grad"), by max or sum."""
        self._ensure_stats()
        reduce_max = 1 if self.split_reduction == "max" else 0
        if self.split_type == "mean_grad":
            g, dim, counts = self.mean.grad, 3, None
        elif self.split_type == "2d_mean_grad":
            g, dim, counts = self.mean_2d_grad, 2, self._aux["counts"]
        else:
            raise NotImplementedError(self.split_type)
        if g is None:
            raise RuntimeError("update_grads needs a backward pass first")
        g = g.contiguous()
        _lib.call("gsx_densify_accumulate", self.N, ptr(g), dim, ptr(counts) if counts is not None else None,
                  ptr(self.grad_mean), reduce_max, stream_handle(self.device))

    @torch.no_grad()
    def split_gaussians(self):
        """gs/sh_renderer.py:426-540: Gaussians whose statistic exceeds
        pos_grad_thresh are split in two (large: any scale above
        split_scale_thresh) or cloned; new arrays are [not split] ++ [clones]
        ++ [split samples, copy 0 then copy 1]."""
        self._ensure_stats()
        n = self.N
        dev = self.device
        cls = torch.empty(n, dtype=torch.uint8, device=dev)
        s = stream_handle(dev)
        _lib.call("gsx_densify_classify", n, ptr(self.grad_mean), ptr(self.cnt),
                  ptr(self.svec_before_activation), float(self.pos_grad_thresh), float(self.split_scale_thresh),
                  1 if self.split_reduction == "mean" else 0, ptr(cls), s)
        stay = (cls != 2).to(torch.int64)
        clone = (cls == 1).to(torch.int64)
        split = (cls == 2).to(torch.int64)
        pos = [torch.cumsum(m, 0) - m for m in (stay, clone, split)]
        n_stay, n_clone, n_split = (int(v) for v in torch.stack([stay.sum(), clone.sum(), split.sum()]).tolist())
        new_n = n_stay + n_clone + 2 * n_split
        sh_len = 3 * self.sh_coeffs.shape[-1]
        out = [torch.empty((new_n, 3), device=dev), torch.empty((new_n, 4), device=dev),
               torch.empty((new_n, 3), device=dev), torch.empty((new_n,) + tuple(self.sh_coeffs.shape[1:]), device=dev),
               torch.empty((new_n,), device=dev)]
        _lib.call("gsx_densify_rewrite", n, ptr(cls), *(ptr(p) for p in pos), n_stay, n_clone, n_split,
                  ptr(self.mean), ptr(self.qvec), ptr(self.svec_before_activation), ptr(self.sh_coeffs), sh_len,
                  ptr(self.alpha_before_activation), float(self.scale_shrink_factor), int(self.split_seed),
                  *(ptr(o) for o in out), s)
        self.split_seed += 1
        self._set_params(*out)
        return n_split, n_clone

    @torch.no_grad()
    def select_masked_gaussians(self, mask):
        """gs/sh_renderer.py:731-741."""
        self._set_params(self.mean.data[mask], self.qvec.data[mask], self.svec_before_activation.data[mask],
                         self.sh_coeffs.data[mask], self.alpha_before_activation.data[mask])

    @torch.no_grad()
    def remove_low_alpha_gaussians(self):
        """gs/sh_renderer.py:542-558: keep opacity >= alpha_thresh."""
        self.select_masked_gaussians(self.alpha >= self.alpha_thresh)

    @torch.no_grad()
    def reset_alpha(self):
        """gs/sh_renderer.py:581-586."""
        v = float(np.log(self.alpha_reset_val / (1.0 - self.alpha_reset_val)))
        self.alpha_before_activation.data.fill_(v)

    def adaptive_control(self, epoch, force=False):
        """gs/sh_renderer.py:626-660."""
        if epoch in self.sh_upgrades:
            self.upgrade_sh()
        if epoch < self.warm_up:
            return
        self.update_grads()

        def step_check(step, size):
            return size != 0 and step != 0 and step % size == 0

        if step_check(epoch, self.adaptive_control_iteration) or force:
            self.split_gaussians()
            self.N_changed = True
        if step_check(epoch, self.remove_low_alpha_period) or force:
            self.remove_low_alpha_gaussians()
            self.N_changed = True
        if step_check(epoch, self.alpha_reset_period) or force:
            self.reset_alpha()
            self.N_changed = True
        if self.N_changed:
            self.grad_mean = torch.zeros(self.N, dtype=torch.float32, device=self.device)
            self.cnt = torch.zeros(self.N, dtype=torch.int32, device=self.device)
            self.N_changed = False

    def _set_params(self, mean, qvec, log_scale, sh, alpha_logit):
        self.mean = torch.nn.Parameter(mean.contiguous())
        self.qvec = torch.nn.Parameter(qvec.contiguous())
        self.svec_before_activation = torch.nn.Parameter(log_scale.contiguous())
        self.sh_coeffs = torch.nn.Parameter(sh.contiguous())
        self.alpha_before_activation = torch.nn.Parameter(alpha_logit.contiguous())
        self.N = int(mean.shape[0])
        self._aux = None

    def upgrade_sh(self):
        """One step of the SH warm-up (gs/sh_renderer.py:625-630)."""
        self.now_C = min(self.now_C + 1, self.max_C)

    def save(self, path):
        """The reference's checkpoint layout (gs/sh_renderer.py:663-679)."""
        save_state(path, self.mean, self.qvec, self.svec_before_activation, self.sh_coeffs,
                   self.alpha_before_activation, self.cfg)

    @classmethod
    def load(cls, path, cfg=None, device="cuda"):
        """Reads checkpoints written by the reference's SHRenderer.save
        (gs/sh_renderer.py:663-708) or by this class; a pickled Hydra/OmegaConf
        configuration loads without omegaconf installed."""
        sd = load_state(path, device)
        C = int(round(sd["sh_coeffs"].shape[-1] ** 0.5))
        saved_cfg = sd.get("cfg")
        use_cfg = cfg if cfg is not None else (saved_cfg if hasattr(saved_cfg, "get") else None)
        r = cls(use_cfg, device=device, sh_order=C)
        r.max_C = C
        r.N = sd["N"]
        for k in PARAM_KEYS:
            setattr(r, k, torch.nn.Parameter(sd[k]))
        return r

    def get_param_groups(self):
        return {"mean": self.mean, "qvec": self.qvec, "svec": self.svec_before_activation,
                "sh_coeffs": self.sh_coeffs, "alpha": self.alpha_before_activation}
