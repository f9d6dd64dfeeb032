"""Batched multi-view passes: one launch per stage for all views.

* images of a batch are bit-identical to rendering each view alone with the
  same tile shape (same per-tile lists, same per-pixel arithmetic);
* batched gradients equal the sum of the per-view gradients within
  1e-4 * max |reference| (only the summation order differs);
* a captured CUDA graph replays to the same images and gradients as the
  eager step and follows in-place parameter updates.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import batch as B  # noqa: E402
from gaussian_splatting_3d_gb300 import renderer, scene as S  # noqa: E402
from gaussian_splatting_3d_gb300.camera import CameraInfo, look_at_c2w, make_gsx_camera  # noqa: E402

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("raster_flags_clean")]
GRAD_REL = 1e-4


def dev():
    return torch.device("cuda:0")


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).max(initial=0.0) / max(np.abs(b).max(initial=0.0), 1e-3))


def make_views(n_views, seed, sizes=((96, 80), (128, 96), (64, 64), (160, 90))):
    dirs = S.sphere_direction(seed, 9, n_views)
    views = []
    for i in range(n_views):
        w, h = sizes[i % len(sizes)]
        cam = CameraInfo.from_vertical_fov(55.0, w, h)
        views.append((look_at_c2w(4.5 * dirs[i]), cam))
    return views


def single_view(scene_t, c2w, cam, W, settings):
    params = [t.clone().requires_grad_(True) for t in
              (scene_t.mean, scene_t.qvec, scene_t.log_scale, scene_t.sh, scene_t.alpha_logit)]
    img = renderer.rasterize(*params, c2w, cam, settings)
    (img * W).sum().backward()
    return img.detach(), [p.grad for p in params]


@pytest.mark.parametrize("tile", [(16, 16), (8, 8), (32, 8)])
def test_batch_matches_per_view(tile):
    sc = S.custom_workload(4000, 64, 64, 3, seed=31).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = make_views(5, seed=31)
    st = renderer.RasterSettings(tile_w=tile[0], tile_h=tile[1])
    bp = B.BatchPipeline(dev(), st).plan([scene_t], [B.ViewSpec(0, c, cam) for c, cam in views])
    rng = np.random.default_rng(0)
    Ws = [torch.from_numpy(rng.random((cam.h, cam.w, 3), dtype=np.float32)).to(dev()) for _, cam in views]
    for g, W in zip(bp.grad_outs, Ws):
        g.copy_(W)
    bp.step()
    torch.cuda.synchronize()
    sums = None
    for i, (c2w, cam) in enumerate(views):
        img, grads = single_view(scene_t, c2w, cam, Ws[i], st)
        np.testing.assert_array_equal(bp.images[i].cpu().numpy(), img.cpu().numpy())
        sums = grads if sums is None else [a + b for a, b in zip(sums, grads)]
    got = [bp.g_mean, bp.g_qvec, bp.g_log_scale, bp.g_sh, bp.g_alpha_logit]
    for name, g, r in zip(["mean", "qvec", "log_scale", "sh", "alpha_logit"], got, sums):
        assert rel_err(g.cpu().numpy(), r.cpu().numpy()) <= GRAD_REL, name


def test_batch_multi_scene_forward():
    scenes_np = [S.custom_workload(n, 64, 64, 3, seed=40 + i).scene for i, n in enumerate((1500, 3000))]
    scenes = [B.Scene.from_arrays(s, dev()) for s in scenes_np]
    views = make_views(4, seed=41)
    specs = [B.ViewSpec(i % 2, c, cam) for i, (c, cam) in enumerate(views)]
    st = renderer.RasterSettings()
    bp = B.BatchPipeline(dev(), st).plan(scenes, specs, backward=False)
    bp.forward()
    torch.cuda.synchronize()
    for i, spec in enumerate(specs):
        s = scenes[spec.scene]
        img = renderer.rasterize(s.mean, s.qvec, s.log_scale, s.sh, s.alpha_logit, spec.c2w, spec.cam, st)
        np.testing.assert_array_equal(bp.images[i].cpu().numpy(), img.cpu().numpy())


def test_batch_graph_replay_matches_eager_and_follows_updates():
    sc = S.custom_workload(3000, 64, 64, 3, seed=51).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = make_views(3, seed=52)
    bp = B.BatchPipeline(dev()).plan([scene_t], [B.ViewSpec(0, c, cam) for c, cam in views])
    for g in bp.grad_outs:
        g.fill_(1.0)
    bp.step()
    eager_imgs = [im.clone() for im in bp.images]
    eager_g = bp.g_sh.clone()
    bp.capture()
    bp.replay()
    for a, b in zip(bp.images, eager_imgs):
        np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    assert rel_err(bp.g_sh.cpu().numpy(), eager_g.cpu().numpy()) <= GRAD_REL
    # the graph reads the live parameter buffers: an in-place update shows up
    with torch.no_grad():
        scene_t.sh[:, :, 0] += 0.5
    bp.replay()
    img_new = renderer.rasterize(scene_t.mean, scene_t.qvec, scene_t.log_scale, scene_t.sh, scene_t.alpha_logit,
                                 views[0][0], views[0][1], renderer.RasterSettings())
    np.testing.assert_array_equal(bp.images[0].cpu().numpy(), img_new.cpu().numpy())


def test_autotuner_picks_a_listed_shape():
    sc = S.custom_workload(2000, 64, 64, 3, seed=61).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = [B.ViewSpec(0, c, cam) for c, cam in make_views(2, seed=62)]
    best, times = B.autotune_tile([scene_t], views, reps=1, device=dev())
    shapes = {(8, 8), (16, 16), (32, 8)}
    assert best in times and set(times) == {(w, h, p) for w, h in shapes for p in (0, 1, 2)}
    assert all(t > 0 for t in times.values())


def test_batched_schedules_give_the_same_images_and_close_gradients():
    """Pixels per thread in the batched raster passes: images bit-identical,
    gradients within the parity tolerance of one another."""
    sc = S.custom_workload(3000, 64, 64, 3, seed=63).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = [B.ViewSpec(0, c, cam) for c, cam in make_views(3, seed=64)]
    runs = []
    for ppt in (1, 2):
        bp = B.BatchPipeline(dev(), renderer.RasterSettings(pixels_per_thread=ppt)).plan([scene_t], views)
        gen = torch.Generator(device="cpu").manual_seed(5)
        for g in bp.grad_outs:
            g.copy_(torch.rand(g.shape, generator=gen))
        bp.step()
        torch.cuda.synchronize()
        runs.append(([im.cpu().numpy() for im in bp.images],
                     [t.cpu().numpy().astype(np.float64) for t in (bp.g_mean, bp.g_qvec, bp.g_log_scale, bp.g_sh,
                                                                   bp.g_alpha_logit)]))
    for a, b in zip(runs[0][0], runs[1][0]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(runs[0][1], runs[1][1]):
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(b).max(), 1e-3)


def test_batch_with_more_than_65536_tiles_matches_per_view():
    """9 views of 1920x1080 at 16x16 tiles: 73,440 tiles, so the global tile
    ids (start/end) take 17 bits while the view-major tile sort runs on the
    13 local bits; every image must still equal the view rendered alone."""
    sc = S.custom_workload(3000, 64, 64, 3, seed=37).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = make_views(9, seed=37, sizes=((1920, 1080),))
    st = renderer.RasterSettings()
    total_tiles = sum(((c.w + 15) // 16) * ((c.h + 15) // 16) for _, c in views)
    assert 1 << 16 < total_tiles <= 1 << 18
    bp = B.BatchPipeline(dev(), st).plan([scene_t], [B.ViewSpec(0, c, cam) for c, cam in views],
                                         backward=False)
    bp.forward()
    torch.cuda.synchronize()
    params = [scene_t.mean, scene_t.qvec, scene_t.log_scale, scene_t.sh, scene_t.alpha_logit]
    for i, (c2w, cam) in enumerate(views):
        img = renderer.rasterize(*params, c2w, cam, st)
        np.testing.assert_array_equal(bp.images[i].cpu().numpy(), img.cpu().numpy())


def test_persistent_raster_matches_one_cta_per_tile():
    """The persistent raster grids (tiles claimed longest first through a
    work counter) give the images of one CTA per tile bit for bit and the
    gradients within the parity tolerance."""
    sc = S.custom_workload(3000, 64, 64, 3, seed=65).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = [B.ViewSpec(0, c, cam) for c, cam in make_views(4, seed=66)]
    runs = []
    for persistent in (False, True):
        bp = B.BatchPipeline(dev(), renderer.RasterSettings(), persistent=persistent).plan([scene_t], views)
        gen = torch.Generator(device="cpu").manual_seed(6)
        for g in bp.grad_outs:
            g.copy_(torch.rand(g.shape, generator=gen))
        bp.step()
        bp.step()  # the counter is zeroed per launch: a second step claims every tile again
        torch.cuda.synchronize()
        runs.append(([im.cpu().numpy() for im in bp.images],
                     [t.cpu().numpy().astype(np.float64) for t in (bp.g_mean, bp.g_qvec, bp.g_log_scale, bp.g_sh,
                                                                   bp.g_alpha_logit)]))
    for a, b in zip(runs[0][0], runs[1][0]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(runs[0][1], runs[1][1]):
        assert np.abs(a - b).max() <= 1e-4 * max(np.abs(b).max(), 1e-3)


def batch_lists(bp, tables):
    """Per view and tile: the batch's list as the view's Gaussian ids."""
    ids, start, end = bp.ids.cpu().numpy(), bp.start.cpu().numpy(), bp.end.cpu().numpy()
    out = []
    for e in tables:
        lists = {}
        for t in range(e.n_tiles_w * e.n_tiles_h):
            g = e.tile_offset + t
            if start[g] >= 0:
                lists[t] = ids[start[g]:end[g]] - e.item_offset
        out.append(lists)
    return out


def test_batch_lists_equal_the_views_own_lists():
    """The view-major batched binning (items ordered by (view, depth), keys
    (view << shift) | local tile, sorted on the local bits) gives every tile
    of every view exactly the list the single-view binning gives it: same
    Gaussians, same depth order."""
    sc = S.custom_workload(6000, 64, 64, 3, seed=71).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = make_views(6, seed=72, sizes=((160, 90), (96, 80), (128, 128)))
    st = renderer.RasterSettings()
    bp = B.BatchPipeline(dev(), st).plan([scene_t], [B.ViewSpec(0, c, cam) for c, cam in views], backward=False)
    bp.forward()
    torch.cuda.synchronize()
    got = batch_lists(bp, [bp.table[i] for i in range(len(views))])
    for i, (c2w, cam) in enumerate(views):
        pr = renderer.project(scene_t.mean, scene_t.qvec, scene_t.log_scale, scene_t.alpha_logit,
                              make_gsx_camera(c2w, cam), st)
        ntw, nth = st.tiles(cam)
        ids, start, end, K = renderer.bin_gaussians(pr, ntw, nth)
        ids, start, end = ids.cpu().numpy(), start.cpu().numpy(), end.cpu().numpy()
        want = {t: ids[start[t]:end[t]] for t in range(ntw * nth) if start[t] >= 0}
        assert set(got[i]) == set(want), i
        for t in want:
            np.testing.assert_array_equal(got[i][t], want[t], err_msg=f"view {i} tile {t}")


def test_batch_of_257_views_takes_global_tile_keys():
    """More than 256 views: the binning keeps global tile ids (no view-major
    pass); images still equal the views rendered alone."""
    sc = S.custom_workload(1500, 64, 64, 3, seed=73).scene
    scene_t = B.Scene.from_arrays(sc, dev())
    views = make_views(257, seed=74, sizes=((32, 32), (48, 32)))
    st = renderer.RasterSettings()
    bp = B.BatchPipeline(dev(), st).plan([scene_t], [B.ViewSpec(0, c, cam) for c, cam in views], backward=False)
    bp.forward()
    torch.cuda.synchronize()
    params = [scene_t.mean, scene_t.qvec, scene_t.log_scale, scene_t.sh, scene_t.alpha_logit]
    for i in range(0, 257, 16):
        c2w, cam = views[i]
        img = renderer.rasterize(*params, c2w, cam, st)
        np.testing.assert_array_equal(bp.images[i].cpu().numpy(), img.cpu().numpy())
