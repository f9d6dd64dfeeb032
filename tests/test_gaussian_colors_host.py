"""The opt-in per-Gaussian colour mode of the FP64 dense restatement
(oracle/fp64_render.py, sh_mode="gaussian"), on the CPU: the colours are
sigmoid(sh . Y(dir)) with dir the unit vector camera centre -> mean, and the
autograd gradient of the rendered image equals central finite differences
(so it can serve as the reference of the CUDA mode)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import scene as S  # noqa: E402
from oracle import fp64_render as R  # noqa: E402


def test_gaussian_colors_formula():
    wl = S.custom_workload(50, 32, 32, 3, seed=61)
    view = wl.views[0]
    cam = R.Cam64.from_view(view.c2w, view.cam)
    mean, _, _, sh, _ = R.to64(wl.scene)
    rgb = R.gaussian_colors(mean, sh, cam, 4).numpy()
    c2w = np.asarray(view.c2w, np.float64).reshape(3, 4)
    d = wl.scene.mean.astype(np.float64) - c2w[:, 3]
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    x, y, z = d.T
    c = R.SH_C
    Y = np.stack([np.full_like(x, c[0]), -c[1] * y, c[1] * z, -c[1] * x, c[2] * x * y, -c[2] * y * z,
                  c[3] * z * z - c[4], -c[2] * x * z, c[5] * (x * x - y * y), c[6] * y * (y * y - 3 * x * x),
                  c[7] * x * y * z, c[8] * y * (1 - 5 * z * z), c[9] * z * (5 * z * z - 3), c[8] * x * (1 - 5 * z * z),
                  c[10] * z * (x * x - y * y), c[6] * x * (3 * y * y - x * x)], -1)
    ref = 1 / (1 + np.exp(-(wl.scene.sh.astype(np.float64) * Y[:, None, :]).sum(-1)))
    np.testing.assert_allclose(rgb, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("mode", ["parity", "exact"])
def test_gaussian_mode_autograd_matches_finite_differences(mode):
    """Central differences on the SH coefficients and the mean of a few
    Gaussians (the colour path's two inputs), through the full render."""
    wl = S.custom_workload(300, 40, 32, 3, seed=67, radius=3.0)
    view = wl.views[0]
    cam = R.Cam64.from_view(view.c2w, view.cam)
    p64 = R.to64(wl.scene)
    W = torch.tensor(wl.grad_weight, dtype=torch.float64)
    st = R.Settings64()
    g, _ = R.param_grads(p64, W, cam, st, 4, mode, sh_mode="gaussian")

    def loss(params):
        return float((R.render(*params, cam, st, 4, mode, sh_mode="gaussian") * W).sum())

    order = torch.argsort(g["sh"].abs().sum((1, 2)), descending=True)[:4].tolist()
    h = 1e-6
    for j in order:
        for name, idx in (("sh", (j, 1, 5)), ("sh", (j, 0, 0)), ("mean", (j, 0)), ("mean", (j, 2))):
            k = ["mean", "qvec", "log_scale", "sh", "alpha_logit"].index(name)
            plus = [p.clone() for p in p64]
            minus = [p.clone() for p in p64]
            plus[k][idx] += h
            minus[k][idx] -= h
            fd = (loss(plus) - loss(minus)) / (2 * h)
            if name == "sh" or mode == "exact":  # parity detaches depth and J, the colour path is exact
                assert abs(fd - float(g[name][idx])) <= 1e-5 * max(1.0, abs(fd)), (name, idx, fd, float(g[name][idx]))


def test_ray_direction_camera_constants():
    """camera_floats(..., "ray") packs the rotation rows so that the raster's
    stride-3 reads give R (x, y, 1); "reference" keeps the flat [3,4]."""
    from gaussian_splatting_3d_gb300 import renderer
    from gaussian_splatting_3d_gb300.camera import CameraInfo, look_at_c2w

    cam = CameraInfo.from_vertical_fov(50.0, 64, 48)
    c2w = look_at_c2w((1.0, -6.0, 2.0))
    ref = renderer.camera_floats(c2w, cam, "reference")[2:]
    ray = renderer.camera_floats(c2w, cam, "ray")[2:]
    np.testing.assert_array_equal(ref, c2w.reshape(-1))
    v = np.array([0.3, -0.2, 1.0], np.float32)
    d = np.array([ray[3 * r] * v[0] + ray[3 * r + 1] * v[1] + ray[3 * r + 2] for r in range(3)])
    np.testing.assert_allclose(d, c2w[:, :3] @ v, rtol=1e-6)
