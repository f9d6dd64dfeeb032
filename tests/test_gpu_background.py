"""Background compositing and output maps (no reference counterpart: the
reference's background variant does not compile; checked against the CPU
oracle and the FP64 reference).

* with a background colour the image equals the oracle's within 2e-6, and
  the alpha (1 - final transmittance) and depth (sum T a G z) maps equal the
  oracle's within 2e-6 and 2e-5 (depths ~ 4);
* gradients with a background (exact mode) equal FP64 autograd of the image
  with the background within 1e-4 * max |reference|;
* without a background the image is bit-identical to the plain path;
* SHRenderer's bg / bg_rgb configuration keys turn it on.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import renderer, scene as S  # noqa: E402
from gaussian_splatting_3d_gb300.sh_renderer import SHRenderer  # noqa: E402
from oracle import fp64_render as R  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("raster_flags_clean")]
BG = (0.2, 0.5, 0.9)
KEYS = ["mean", "qvec", "log_scale", "sh", "alpha_logit"]


def dev():
    return torch.device("cuda:0")


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max(initial=0.0) / max(np.abs(b).max(initial=0.0), 1e-3))


def params_of(sc, grad=False):
    return [torch.from_numpy(a).to(dev()).requires_grad_(grad) for a in
            (sc.mean, sc.qvec, sc.log_scale, sc.sh, sc.alpha_logit)]


def test_background_and_maps_match_oracle():
    wl = S.custom_workload(5000, 100, 72, 3, seed=12, radius=3.5)  # some tiles left empty
    sc, view = wl.scene, wl.views[0]
    ref = O.render_view(sc, view, bg=BG)
    aux = {}
    img = renderer.rasterize(*params_of(sc), view.c2w, view.cam,
                             renderer.RasterSettings(bg=BG, output_maps=True), aux)
    np.testing.assert_allclose(img.cpu().numpy(), ref["image"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(aux["alpha_map"].cpu().numpy(), ref["alpha_map"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(aux["depth_map"].cpu().numpy(), ref["depth_map"], rtol=0, atol=2e-5)
    assert float(aux["alpha_map"].min()) == 0.0 and float(aux["alpha_map"].max()) > 0.5
    plain = renderer.rasterize(*params_of(sc), view.c2w, view.cam, renderer.RasterSettings())
    plain_maps = renderer.rasterize(*params_of(sc), view.c2w, view.cam, renderer.RasterSettings(output_maps=True))
    np.testing.assert_array_equal(plain.cpu().numpy(), plain_maps.cpu().numpy())


def test_background_gradients_exact():
    wl = S.diff_workload(log_scale_mu=-2.5)
    sc, view = wl.scene, wl.views[0]
    ps = params_of(sc, grad=True)
    W = torch.from_numpy(wl.grad_weight).to(dev())
    img = renderer.rasterize(*ps, view.c2w, view.cam, renderer.RasterSettings(bg=BG, exact_grad=True))
    (img * W).sum().backward()
    cam = R.Cam64.from_view(view.c2w, view.cam, device=dev())
    ref, img64 = R.param_grads(R.to64(sc, dev()), W.double(), cam, R.Settings64(), sc.sh_order, "exact", bg=BG)
    assert float((img.detach().double() - img64).abs().max()) <= 4e-6
    for k, p in zip(KEYS, ps):
        e = rel_err(p.grad.cpu().numpy(), ref[k].cpu().numpy())
        assert e <= 1e-4, f"{k}: {e:.3g}"


def test_shrenderer_bg_config():
    wl = S.custom_workload(2000, 64, 48, 1, seed=5)
    sc, view = wl.scene, wl.views[0]
    r = SHRenderer({"sh_order": 2, "bg": True, "bg_rgb": list(BG)}, device=dev())
    r._set_params(*params_of(sc))
    r.now_C = 2
    r.eval()
    img = r(view.c2w, view.cam)
    ref = O.render_view(sc, view, bg=BG)["image"]
    np.testing.assert_allclose(img.detach().cpu().numpy(), ref, rtol=0, atol=2e-6)
