"""Adaptive density control against the reference's own policy
(tests/golden/densify_400.npz, made by running gs/sh_renderer.py's
update_grads / split_gaussians / remove_low_alpha_gaussians here).

* the gradient statistic (max or sum of |dL/dmean| or of |dL/dmean2d| over
  the visible Gaussians) equals the reference's within 1e-6 relative;
* split / clone produce the reference's Gaussian count and arrays: the
  Gaussians that stay and the clones bit for bit, the split copies with the
  source's rotation, SH and opacity, log-scale log(scale / 1.6), and means
  mean + R^T (n * scale) with n standard normal (the reference draws n with
  torch.randn, this package with its own generator, so n is checked for its
  distribution);
* the low-opacity prune keeps the reference's count and rows.
"""
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300.sh_renderer import SHRenderer  # noqa: E402

pytestmark = pytest.mark.gpu
FIX = Path(__file__).parent / "golden" / "densify_400.npz"
CASES = [(t, r) for t in ("mean_grad", "2d_mean_grad") for r in ("max", "mean")]


def dev():
    return torch.device("cuda:0")


def quat_rot(q):
    q = q / np.maximum(np.linalg.norm(q, axis=-1, keepdims=True), 1e-12)
    w, x, y, z = q.T
    return np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                     2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                     2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1).reshape(-1, 3, 3)


@pytest.mark.parametrize("split_type,red", CASES)
def test_density_control_matches_reference(split_type, red):
    f = dict(np.load(FIX))
    n = f["mean"].shape[0]
    cfg = {"sh_order": 4, "split_type": split_type, "split_reduction": red, "pos_grad_thresh": float(f["thresh"]),
           "split_scale_thresh": float(f["scale_thresh"]), "scale_shrink_factor": float(f["shrink"]),
           "alpha_thresh": 0.3}
    r = SHRenderer(cfg, device=dev())
    r._set_params(*(torch.from_numpy(f[k]).to(dev()) for k in ("mean", "qvec", "log_scale", "sh", "alpha_logit")))
    r.grad_mean = torch.from_numpy(f["gm0"]).to(dev())
    r.cnt = torch.from_numpy(f["cnt0"]).to(dev())
    r.mean.grad = torch.from_numpy(f["G3"]).to(dev())
    r._aux = {"counts": torch.from_numpy(f["vis"].astype(np.int32)).to(dev()),
              "mean2d_grad": torch.from_numpy(f["G2"] * f["vis"][:, None]).to(dev())}
    tag = f"{split_type}_{red}"
    r.update_grads()
    gm = r.grad_mean.cpu().numpy()
    np.testing.assert_allclose(gm, f[f"grad_mean_{tag}"], rtol=1e-6, atol=0)

    n_split, n_clone = r.split_gaussians()
    assert r.N == int(f[f"split_{tag}_N"]) == n + n_split + n_clone
    got = {k: getattr(r, k).data.cpu().numpy() for k in
           ("mean", "qvec", "svec_before_activation", "sh_coeffs", "alpha_before_activation")}
    ref = {k: f[f"split_{tag}_{k}"] for k in got}
    head = n - n_split + n_clone  # the Gaussians that stay, then the clones
    for k in got:
        np.testing.assert_array_equal(got[k][:head], ref[k][:head])
    for k in ("qvec", "sh_coeffs", "alpha_before_activation"):
        np.testing.assert_array_equal(got[k][head:], ref[k][head:])
    np.testing.assert_allclose(got["svec_before_activation"][head:], ref["svec_before_activation"][head:],
                               rtol=0, atol=2e-6)
    # split copies: mean = source + R^T (n * scale)
    stat = gm / (f["cnt0"] + 1e-5) if red == "mean" else gm
    chosen = stat > f["thresh"]
    large = (np.exp(f["log_scale"].astype(np.float64)) > f["scale_thresh"]).any(-1)
    src = np.nonzero(chosen & large)[0]
    assert len(src) == n_split > 20
    s = np.exp(f["log_scale"][src].astype(np.float64))
    R = quat_rot(f["qvec"][src].astype(np.float64))
    draws = []
    for copy in range(2):
        m_new = got["mean"][head + copy * n_split: head + (copy + 1) * n_split].astype(np.float64)
        d = m_new - f["mean"][src]
        draws.append(np.einsum("bij,bj->bi", R, d) / s)  # R (R^T (n s)) / s = n
    draws = np.concatenate(draws).ravel()
    assert np.all(np.isfinite(draws)) and np.abs(draws).max() < 6.5
    assert abs(draws.mean()) < 0.25 and 0.8 < draws.std() < 1.2

    r.remove_low_alpha_gaussians()
    assert r.N == int(f[f"prune_{tag}_N"])
    keep_head = int((1 / (1 + np.exp(-ref["alpha_before_activation"][:head].astype(np.float64))) >= 0.3).sum())
    np.testing.assert_array_equal(r.mean.data.cpu().numpy()[:keep_head], f[f"prune_{tag}_mean"][:keep_head])


def test_forward_counts_visits_and_exposes_mean2d_grad():
    from gaussian_splatting_3d_gb300 import scene as S

    wl = S.custom_workload(3000, 96, 80, 3, seed=3, radius=2.0)  # close: some Gaussians culled
    sc, view = wl.scene, wl.views[0]
    r = SHRenderer({"sh_order": 4, "split_type": "2d_mean_grad"}, device=dev())
    r._set_params(*(torch.from_numpy(a).to(dev()) for a in (sc.mean, sc.qvec, sc.log_scale, sc.sh, sc.alpha_logit)))
    r.now_C = 4
    r.train()
    for _ in range(2):
        img = r(view.c2w, view.cam)
        (img * torch.from_numpy(wl.grad_weight).to(dev())).sum().backward()
        r.update_grads()
    vis = r.frustum_culling_mask
    assert 0 < int(vis.sum()) < sc.n
    np.testing.assert_array_equal(r.cnt.cpu().numpy(), 2 * vis.cpu().numpy().astype(np.int32))
    g2 = r.mean_2d_grad
    assert g2.shape == (sc.n, 2) and float(g2[~vis].abs().max()) == 0.0
    expect = torch.linalg.vector_norm(g2, dim=-1)  # the same gradient both steps: max = one norm
    torch.testing.assert_close(r.grad_mean, expect, rtol=1e-6, atol=0)
