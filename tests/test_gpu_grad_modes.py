"""Gradient modes of the CUDA backward on the differentiation workload
(2,000 Gaussians, 64x64, SH degree 1; and a variant with larger, opaque
Gaussians where the 0.99 opacity clamp and the transmittance cut-off act).

* In every mode (parity = the reference's gradient, depth =
  depth_detach=False, exact = the true derivative) the CUDA gradients of
  sum(W * image) through the autograd Function equal the FP64 dense
  reference's autograd gradients within 1e-4 * max |reference| per tensor.
* Exact mode against central finite differences in FP64 (step 1e-4) on every
  parameter of 200 randomly chosen Gaussians: within 1e-4 * max |FD| per
  parameter group, on the entries where the step 1e-4 and 5e-5 estimates
  agree (the others straddle a discontinuity of the renderer).
* The batched backward in exact mode equals the sum of per-view exact
  gradients.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import batch as B  # noqa: E402
from gaussian_splatting_3d_gb300 import renderer, scene as S  # noqa: E402
from oracle import fp64_render as R  # noqa: E402

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("raster_flags_clean")]
GRAD_REL = 1e-4
KEYS = ["mean", "qvec", "log_scale", "sh", "alpha_logit"]
WORKLOADS = {"diff": {}, "diff_clamp": dict(log_scale_mu=-2.0, alpha_mu=3.0)}
SETTINGS = {"parity": dict(), "depth": dict(depth_detach=False), "exact": dict(exact_grad=True)}


def dev():
    return torch.device("cuda:0")


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max(initial=0.0) / max(np.abs(b).max(initial=0.0), 1e-3))


def cuda_grads(wl, mode):
    sc, view = wl.scene, wl.views[0]
    ps = [torch.from_numpy(a).to(dev()).requires_grad_(True) for a in
          (sc.mean, sc.qvec, sc.log_scale, sc.sh, sc.alpha_logit)]
    img = renderer.rasterize(*ps, view.c2w, view.cam, renderer.RasterSettings(**SETTINGS[mode]))
    (img * torch.from_numpy(wl.grad_weight).to(dev())).sum().backward()
    return {k: p.grad.double() for k, p in zip(KEYS, ps)}, img.detach()


def fp64_setup(wl):
    view = wl.views[0]
    cam = R.Cam64.from_view(view.c2w, view.cam, device=dev())
    W = torch.tensor(wl.grad_weight, dtype=torch.float64, device=dev())
    return R.to64(wl.scene, dev()), cam, W


@pytest.mark.parametrize("name", list(WORKLOADS))
@pytest.mark.parametrize("mode", list(SETTINGS))
def test_cuda_gradients_match_fp64_autograd(name, mode):
    wl = S.diff_workload(**WORKLOADS[name])
    got, img = cuda_grads(wl, mode)
    p64, cam, W = fp64_setup(wl)
    ref, img64 = R.param_grads(p64, W, cam, R.Settings64(), wl.scene.sh_order, mode)
    assert float((img.double() - img64).abs().max()) <= 4e-6
    for k in KEYS:
        e = rel_err(got[k].cpu().numpy(), ref[k].cpu().numpy())
        assert e <= GRAD_REL, f"{mode} {k}: {e:.3g}"


def test_exact_backward_against_finite_differences():
    """Config 4a: every parameter of 200 random Gaussians of 2,000."""
    wl = S.diff_workload()
    C = wl.scene.sh_order
    got, _ = cuda_grads(wl, "exact")
    p64, cam, W = fp64_setup(wl)
    js = np.random.default_rng(2024).choice(wl.scene.n, 200, replace=False)
    rows, fds, stables = [], [], []
    for j in js:
        fh, fh2 = R.fd_gaussian(p64, W, cam, R.Settings64(), C, int(j), h=1e-4)
        an = R.gaussian_param_rows(got, int(j), C)
        scale = max(float(fh.abs().max()), 1e-3)
        rows.append(an)
        fds.append(fh)
        stables.append((fh - fh2).abs() <= 1e-6 * scale + 1e-9)
    an = torch.stack(rows).cpu().numpy()
    fd = torch.stack(fds).cpu().numpy()
    ok = torch.stack(stables).cpu().numpy()
    assert ok.mean() >= 0.95, f"only {ok.mean():.3f} of the FD entries are stable"
    groups = {"mean": slice(0, 3), "qvec": slice(3, 7), "log_scale": slice(7, 10),
              "sh": slice(10, 10 + 3 * C * C), "alpha_logit": slice(10 + 3 * C * C, 11 + 3 * C * C)}
    assert np.abs(fd).max() > 0.1  # the chosen Gaussians do contribute
    for k, sl in groups.items():
        a, f, m = an[:, sl], fd[:, sl], ok[:, sl]
        e = float((np.abs(a - f) * m).max() / max(np.abs(f * m).max(), 1e-3))
        assert e <= GRAD_REL, f"{k}: {e:.3g}"


def test_batched_exact_mode_sums_per_view_exact():
    wl = S.diff_workload(log_scale_mu=-2.5)
    sc = B.Scene.from_arrays(wl.scene, dev())
    dirs = S.sphere_direction(3, 9, 3)
    from gaussian_splatting_3d_gb300.camera import look_at_c2w
    views = [B.ViewSpec(0, look_at_c2w(4.0 * d), wl.views[0].cam) for d in dirs]
    st = renderer.RasterSettings(exact_grad=True)
    bp = B.BatchPipeline(dev(), st).plan([sc], views)
    for g in bp.grad_outs:
        g.fill_(1.0)
    bp.step()
    torch.cuda.synchronize()
    sums = None
    for v in views:
        ps = [t.clone().requires_grad_(True) for t in (sc.mean, sc.qvec, sc.log_scale, sc.sh, sc.alpha_logit)]
        renderer.rasterize(*ps, v.c2w, v.cam, st).sum().backward()
        gs = [p.grad for p in ps]
        sums = gs if sums is None else [a + b for a, b in zip(sums, gs)]
    got = [bp.g_mean, bp.g_qvec, bp.g_log_scale, bp.g_sh, bp.g_alpha_logit]
    for k, g, r in zip(KEYS, got, sums):
        assert rel_err(g.cpu().numpy(), r.cpu().numpy()) <= GRAD_REL, k


def test_recompute_projection_matches_stored():
    """Memory mode (projection re-run in backward, nothing but the tile lists
    held): the same image and the same gradients as with the stored
    projection (the raster backward sums with atomics, hence the tolerance)."""
    wl = S.custom_workload(20000, 160, 120, 3, seed=9)
    sc, view = wl.scene, wl.views[0]
    W = torch.from_numpy(wl.grad_weight).to(dev())
    res = {}
    for rec in (False, True):
        ps = [torch.from_numpy(a).to(dev()).requires_grad_(True) for a in
              (sc.mean, sc.qvec, sc.log_scale, sc.sh, sc.alpha_logit)]
        img = renderer.rasterize(*ps, view.c2w, view.cam, renderer.RasterSettings(recompute_projection=rec))
        (img * W).sum().backward()
        res[rec] = (img.detach().cpu().numpy(), [p.grad.cpu().numpy() for p in ps])
    np.testing.assert_array_equal(res[True][0], res[False][0])
    for k, a, b in zip(KEYS, res[True][1], res[False][1]):
        assert rel_err(a, b) <= 1e-6, k
