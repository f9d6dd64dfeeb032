"""Property tests of the oracle on generated inputs (hypothesis, CPU only).

* binning: the oracle's lists equal an independent statement of the
  reference's order -- every (tile, Gaussian) pair of the AABB rectangles
  sorted by (tile id, depth bits as unsigned) with equal keys in index order
  (np.lexsort) -- with start/end at the tile runs, for rectangles, culled
  Gaussians and depths drawn to collide;
* projection: a visible Gaussian's key count is its rectangle's area and the
  rectangle lies in the tile grid; a culled one has no keys;
* raster forward: every pixel lies in [0, 1] (colours are sigmoids and the
  weights sum to 1 - T) and pixels with no tile list stay 0;
* raster backward: linear in dL/dimage.
"""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from gaussian_splatting_3d_gb300 import scene as S  # noqa: E402
from gaussian_splatting_3d_gb300.camera import frustum_np  # noqa: E402
from oracle import oracle as O  # noqa: E402

SETTINGS = settings(max_examples=40, deadline=None)


def lexsort_lists(rect, depth, ntw, nth):
    tiles, bits, gids = [], [], []
    dbits = np.asarray(depth, np.float32).view(np.uint32)
    for g, (x0, y0, x1, y1) in enumerate(rect):
        for tx in range(x0, x1 + 1):
            for ty in range(y0, y1 + 1):
                tiles.append(ty * ntw + tx)
                bits.append(dbits[g])
                gids.append(g)
    tiles, bits, gids = np.array(tiles, np.int64), np.array(bits, np.int64), np.array(gids, np.int64)
    order = np.lexsort((gids, bits, tiles))
    ids, tiles = gids[order], tiles[order]
    start = np.full(ntw * nth, -1, np.int32)
    end = np.full(ntw * nth, -1, np.int32)
    for t in np.unique(tiles):
        where = np.nonzero(tiles == t)[0]
        start[t], end[t] = where[0], where[-1] + 1
    return ids.astype(np.int32), start, end


@st.composite
def binning_inputs(draw):
    ntw = draw(st.integers(1, 9))
    nth = draw(st.integers(1, 7))
    n = draw(st.integers(0, 60))
    rect = np.zeros((n, 4), np.int32)
    for g in range(n):
        if draw(st.booleans()) and draw(st.integers(0, 4)) == 0:
            rect[g] = (0, 0, -1, -1)  # culled
            continue
        x0 = draw(st.integers(0, ntw - 1))
        y0 = draw(st.integers(0, nth - 1))
        rect[g] = (x0, y0, draw(st.integers(x0, ntw - 1)), draw(st.integers(y0, nth - 1)))
    pool = [1.5, 2.0, 2.0000002, 7.25, 1e3]
    depth = np.array([draw(st.one_of(st.sampled_from(pool),
                                     st.floats(0.0625, 8192.0, allow_nan=False, width=32))) for _ in range(n)],
                     np.float32)
    return rect, depth, ntw, nth


@SETTINGS
@given(binning_inputs())
def test_binning_equals_lexsort_statement(inp):
    rect, depth, ntw, nth = inp
    got = O.bin_gaussians(rect, rect[:, 2:], depth, nth, ntw, stride=4)
    ids, start, end = lexsort_lists(rect, depth, ntw, nth)
    assert got["K"] == len(ids)
    np.testing.assert_array_equal(got["ids"][:got["K"]], ids)
    np.testing.assert_array_equal(got["start"], start)
    np.testing.assert_array_equal(got["end"], end)


def oracle_projection(wl):
    sc, view = wl.scene, wl.views[0]
    cam = view.cam
    normals, pts = frustum_np(view.c2w, cam)
    ocam = O.make_camera(view.c2w, cam.fx, cam.fy, cam.cx, cam.cy, cam.w, cam.h, normals, pts)
    return O.project(sc.mean, sc.qvec, sc.log_scale, sc.alpha_logit, ocam, 1.0, 6.0, view.tile, view.tile)


scenes = st.builds(lambda n, w, h, deg, seed, mu: S.custom_workload(n, w, h, deg, seed=seed, log_scale_mu=mu),
                   st.integers(1, 400), st.integers(16, 96), st.integers(16, 72), st.integers(0, 3),
                   st.integers(0, 10_000), st.sampled_from([-3.5, -3.0, -2.0]))


@SETTINGS
@given(scenes)
def test_projection_counts_are_rectangle_areas(wl):
    pr = oracle_projection(wl)
    view = wl.views[0]
    ntw = (view.cam.w + view.tile - 1) // view.tile
    nth = (view.cam.h + view.tile - 1) // view.tile
    r, c = pr["rect"], pr["counts"]
    vis = c > 0
    area = (r[:, 2] - r[:, 0] + 1) * (r[:, 3] - r[:, 1] + 1)
    np.testing.assert_array_equal(c[vis], area[vis])
    assert np.all((r[vis, 0] >= 0) & (r[vis, 2] < ntw) & (r[vis, 1] >= 0) & (r[vis, 3] < nth))
    assert np.all(c[~vis] == 0)


@settings(max_examples=15, deadline=None)
@given(scenes, st.integers(0, 2 ** 31 - 1))
def test_forward_bounds_and_backward_linearity(wl, seed):
    sc, view = wl.scene, wl.views[0]
    cam = view.cam
    pr = oracle_projection(wl)
    ntw = (cam.w + view.tile - 1) // view.tile
    nth = (cam.h + view.tile - 1) // view.tile
    b = O.bin_gaussians(pr["rect"], pr["rect"][:, 2:], pr["depth"], nth, ntw, stride=4)
    P = O.raster_params(cam.w, cam.h, view.tile, view.tile, sc.sh_order, sc.sh.shape[-1])
    args = (pr["mean2d"], pr["cov2d"], sc.sh, pr["alpha"], b["start"], b["end"], b["ids"],
            np.array(cam.topleft(), np.float32), view.c2w, np.float32(1 / cam.fx), np.float32(1 / cam.fy))
    img = O.render_fwd(P, *args)
    assert np.all(img >= 0.0) and np.all(img <= 1.0 + 1e-6)
    empty = (b["start"] < 0).reshape(nth, ntw)
    mask = np.repeat(np.repeat(empty, view.tile, 0), view.tile, 1)[:cam.h, :cam.w]
    assert np.all(img[mask] == 0.0)
    rng = np.random.default_rng(seed)
    W1 = rng.random(img.shape, dtype=np.float32)
    W2 = rng.random(img.shape, dtype=np.float32)
    g1 = O.render_bwd(P, *args, img, W1)
    g2 = O.render_bwd(P, *args, img, W2)
    g3 = O.render_bwd(P, *args, img, (W1 + 2.0 * W2).astype(np.float32))
    for k in ("mean2d", "cov2d", "alpha", "sh"):
        lin = g1[k].astype(np.float64) + 2.0 * g2[k].astype(np.float64)
        scale = max(np.abs(lin).max(initial=0.0), 1e-3)
        assert np.abs(g3[k] - lin).max(initial=0.0) <= 1e-4 * scale, k
