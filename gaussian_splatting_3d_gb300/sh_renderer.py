"""``SHRenderer`` with the reference's model surface (gs/sh_renderer.py:44-324,
663-729) on the fused sm_103a path.

Same parameter tensors and names (``mean``, ``qvec``, ``svec_before_activation``,
``sh_coeffs``, ``alpha_before_activation``), same activations (exp scales,
sigmoid opacity), same SH warm-up counter ``now_C``, same checkpoint format
(``save`` / ``load``) and ``forward(c2w, camera_info) -> [H, W, 3]``.  The
forward is one fused projection + binning + raster; ``loss.backward()`` runs
the raster backward and the projection backward and fills all five ``.grad``
tensors.  Densification and optimiser policy are outside the rendering path
and are not reproduced.
"""
from __future__ import annotations

from pathlib import Path

import torch

from .camera import CameraInfo
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
            exact_grad=bool(get("exact_grad", False)))
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
        return rasterize(self.mean, self.qvec, self.svec_before_activation, self.sh_coeffs,
                         self.alpha_before_activation, c2w, camera_info, st)

    def upgrade_sh(self):
        """One step of the SH warm-up (gs/sh_renderer.py:625-630)."""
        self.now_C = min(self.now_C + 1, self.max_C)

    def save(self, path):
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        torch.save({"mean": self.mean.data, "qvec": self.qvec.data,
                    "svec_before_activation": self.svec_before_activation.data,
                    "sh_coeffs": self.sh_coeffs.data,
                    "alpha_before_activation": self.alpha_before_activation.data,
                    "N": self.N, "cfg": self.cfg}, path)

    @classmethod
    def load(cls, path, cfg=None, device="cuda"):
        """Reads checkpoints written by the reference's SHRenderer.save
        (gs/sh_renderer.py:663-708) or by this class."""
        sd = torch.load(path, map_location=device, weights_only=False)
        r = cls(cfg if cfg is not None else sd.get("cfg"), device=device,
                sh_order=int(round(sd["sh_coeffs"].shape[-1] ** 0.5)))
        r.max_C = int(round(sd["sh_coeffs"].shape[-1] ** 0.5))
        r.N = int(sd["N"])
        for k in ("mean", "qvec", "svec_before_activation", "sh_coeffs", "alpha_before_activation"):
            setattr(r, k, torch.nn.Parameter(sd[k].to(device, torch.float32).contiguous()))
        assert r.N == r.mean.shape[0]
        return r

    def get_param_groups(self):
        return {"mean": self.mean, "qvec": self.qvec, "svec": self.svec_before_activation,
                "sh_coeffs": self.sh_coeffs, "alpha": self.alpha_before_activation}
