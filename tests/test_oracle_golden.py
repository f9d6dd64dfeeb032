"""The oracle against outputs of the reference itself (tests/golden/*.npz,
made by tests/golden/make_golden.py from the reference's Python and its CUDA
kernels run under CPU emulation).  Each stage is fed the reference's own
inputs for that stage, so a mismatch points at one function.

Tolerances (FP32): culling masks, AABB rectangles, K, start/end and the sorted
id lists (after canonicalising runs of equal keys by index) are compared
exactly.  Projection outputs: relative 1e-5.  Images: max-abs 1e-4 -- the
oracle's exp is gsx_expf, the reference's is libm's expf here (CUDA's on a
GPU), so a pixel may differ by more only where an ulp flips a 1/255 or
T-threshold decision; such flips are counted and must stay below 1 in 10^4
pixels.  Gradients: max |oracle - reference| <= 1e-4 * max |reference| per
tensor (scale floored at 1e-3).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = sorted(p for p in (Path(__file__).parent / "golden").glob("*.npz") if not p.stem.startswith("densify"))
IMG_TOL = 1e-4
GRAD_REL = 1e-4


def load(path):
    d = np.load(path)
    return {k: d[k] for k in d.files}


def rel_err(a, b):
    """max |a - b| / max(max |b|, 1e-3): the floor keeps gradients that are
    analytically zero (pure rounding noise on both sides) from failing."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max(initial=0.0) / max(np.abs(b).max(initial=0.0), 1e-3))


def ocam_of(f):
    fx, fy, cx, cy, w, h = f["cam"]
    return O.make_camera(f["c2w"], fx, fy, cx, cy, int(w), int(h), f["frustum_normals"], f["frustum_pts"])


def dims(f):
    w, h = int(f["cam"][4]), int(f["cam"][5])
    t = int(f["tile"])
    return w, h, t, (w + t - 1) // t, (h + t - 1) // t


@pytest.fixture(params=GOLDEN, ids=[p.stem for p in GOLDEN])
def fx(request):
    return load(request.param)


def test_fixtures_present():
    names = {p.stem for p in GOLDEN}
    assert "small_10k_256_C1" in names and len(names) >= 5


def test_frustum_planes(fx):
    from gaussian_splatting_3d_gb300.camera import CameraInfo, frustum_np

    fxx, fy, cx, cy, w, h = fx["cam"]
    cam = CameraInfo(fxx, fy, cx, cy, int(w), int(h), 1.5, 1000.0)
    n, p = frustum_np(fx["c2w"], cam)
    np.testing.assert_allclose(n, fx["frustum_normals"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(p, fx["frustum_pts"], rtol=0, atol=1e-4)


def test_culling(fx):
    mask = O.cull_bsphere(fx["mean"], fx["svec"], fx["frustum_normals"], fx["frustum_pts"], 1.0)
    np.testing.assert_array_equal(mask, fx["mask"])


def test_projection(fx):
    w, h, t, ntw, nth = dims(fx)
    pr = O.project(fx["mean"], fx["qvec"], fx["svec"], fx["alpha_logit"], ocam_of(fx), 1.0, 6.0, t, t,
                   scales_are_svec=True)
    m = fx["mask"]
    np.testing.assert_array_equal(pr["mask"], m)
    assert rel_err(pr["mean2d"][m], fx["mean2d"]) <= 1e-5
    assert rel_err(pr["cov2d"][m], fx["cov2d"]) <= 1e-5
    assert rel_err(pr["depth"][m], fx["depth"]) <= 1e-6
    assert rel_err(pr["alpha"][m], fx["alpha"]) <= 1e-6
    rect = pr["rect"][m]
    flips = np.any(rect[:, :2] != fx["aabb_tl"], axis=1) | np.any(rect[:, 2:] != fx["aabb_br"], axis=1)
    assert flips.sum() <= max(1, m.sum() // 10000), f"{flips.sum()} AABB rectangles differ"
    if flips.sum() == 0:
        assert int(pr["counts"].sum()) == int(fx["K"])


def test_binning(fx):
    w, h, t, ntw, nth = dims(fx)
    b = O.bin_gaussians(fx["aabb_tl"], fx["aabb_br"], fx["depth"], nth, ntw)
    assert b["K"] == int(fx["K"])
    np.testing.assert_array_equal(b["ids"], fx["ids"])
    np.testing.assert_array_equal(b["start"], fx["start"])
    np.testing.assert_array_equal(b["end"], fx["end"])


def _raster_inputs(fx):
    w, h, t, ntw, nth = dims(fx)
    C = int(fx["now_C"])
    sh_used = np.ascontiguousarray(fx["sh"][fx["mask"]][..., :C * C])
    P = O.raster_params(w, h, t, t, C, C * C)
    return P, sh_used


def test_raster_forward(fx):
    P, sh_used = _raster_inputs(fx)
    img = O.render_fwd(P, fx["mean2d"], fx["cov2d"], sh_used, fx["alpha"], fx["start"], fx["end"], fx["ids_raw"],
                       fx["topleft"], fx["c2w"], fx["psx"], fx["psy"])
    d = np.abs(img - fx["image"]).max(axis=-1)
    over = int((d > IMG_TOL).sum())
    assert over <= max(1, d.size // 10000), f"{over} pixels over {IMG_TOL} (max {d.max():.3g})"
    assert float(np.median(d)) <= 1e-6


def test_raster_backward(fx):
    P, sh_used = _raster_inputs(fx)
    g = O.render_bwd(P, fx["mean2d"], fx["cov2d"], sh_used, fx["alpha"], fx["start"], fx["end"], fx["ids_raw"],
                     fx["topleft"], fx["c2w"], fx["psx"], fx["psy"], fx["image"], fx["grad_weight"])
    C = int(fx["now_C"])
    ref_sh = fx["grad_sh"][fx["mask"]][..., :C * C]
    for k, ref in (("mean2d", fx["g_mean2d"]), ("cov2d", fx["g_cov2d"]), ("alpha", fx["g_alpha"]), ("sh", ref_sh)):
        e = rel_err(g[k], ref)
        assert e <= GRAD_REL, f"{k}: {e:.3g}"


def test_projection_backward(fx):
    m = fx["mask"]
    n = m.shape[0]

    def scatter(a, width):
        out = np.zeros((n, width), np.float32) if width else np.zeros(n, np.float32)
        out[m] = a
        return out

    gp = O.project_bwd(fx["mean"], fx["qvec"], fx["log_scale"], fx["alpha_logit"], ocam_of(fx), m,
                       scatter(fx["g_mean2d"], 2), scatter(fx["g_cov2d"], 4), scatter(fx["g_alpha"], 0))
    for k, ref in (("mean", fx["grad_mean"]), ("qvec", fx["grad_qvec"]), ("log_scale", fx["grad_log_scale"]),
                   ("alpha_logit", fx["grad_alpha_logit"])):
        e = rel_err(gp[k], ref)
        assert e <= GRAD_REL, f"{k}: {e:.3g}"


def test_full_oracle_pipeline_image(fx):
    """Oracle end to end from the parameters (its own projection and binning).
    Where the reference's list holds equal keys in a scheduling-dependent
    order (ids_raw differs from the canonical order), its image depends on
    that order; test_raster_forward covers those fixtures with the
    reference's own order."""
    if not np.array_equal(fx["ids"], fx["ids_raw"]):
        pytest.skip("reference composited equal keys in a non-canonical order")
    from gaussian_splatting_3d_gb300 import scene as S
    from gaussian_splatting_3d_gb300.camera import CameraInfo

    fxx, fy, cx, cy, w, h = fx["cam"]
    cam = CameraInfo(fxx, fy, cx, cy, int(w), int(h), 1.5, 1000.0)
    sc = S.Scene(fx["mean"], fx["qvec"], fx["log_scale"], fx["sh"], fx["alpha_logit"], int(fx["sh_order"]))
    r = O.render_view(sc, S.View(fx["c2w"], cam, int(fx["tile"])), fx["grad_weight"], sh_order=int(fx["now_C"]))
    d = np.abs(r["image"] - fx["image"]).max(axis=-1)
    over = int((d > IMG_TOL).sum())
    assert over <= max(2, d.size // 5000), f"{over} pixels over {IMG_TOL}"
    for k, ref in (("mean", fx["grad_mean"]), ("qvec", fx["grad_qvec"]), ("log_scale", fx["grad_log_scale"]),
                   ("sh", fx["grad_sh"]), ("alpha_logit", fx["grad_alpha_logit"])):
        assert rel_err(r["param_grads"][k], ref) <= 10 * GRAD_REL, k


def test_exp_against_libm():
    xs = np.linspace(-86.9, 88.6, 20001).astype(np.float32)
    got = np.array([O.expf(x) for x in xs], np.float64)
    ref = np.exp(xs.astype(np.float64))
    ulp = np.abs(got - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert ulp.max() < 1.0
