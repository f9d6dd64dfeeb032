"""Tile lists at the largest sizes of the radix sorts, bit for bit against
the oracle.

* the headline view (1,000,000 Gaussians, 1920x1080, 16x16 tiles) binned
  with a key capacity of 40 Mi: the tile sort's grid covers ~13,000 chunks
  of which the ~4.2 M keys fill the first ~1,400, and its lists must equal
  those binned at a capacity near K and the oracle's;
* 34 Mi synthetic Gaussians, one tile each, depths on a coarse grid (many
  equal depth bits per tile, so stability shows): a 32-bit depth sort of
  34 Mi keys and a tile sort of 34 Mi keys, once with 13-bit tile ids (two
  8-bit passes) and once with 17-bit ones (two 9-bit passes).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import renderer, scene as S  # noqa: E402
from gaussian_splatting_3d_gb300.camera import make_gsx_camera  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = [pytest.mark.gpu, pytest.mark.usefixtures("raster_flags_clean")]

LARGE_KEYS = 32 << 20


def bin_and_release(pr, ntw, nth, key_hint):
    try:
        ids, start, end, K = renderer.bin_gaussians(pr, ntw, nth, key_hint=key_hint)
        return ids.cpu().numpy(), start.cpu().numpy(), end.cpu().numpy(), K
    finally:
        renderer._bin_buffers(pr.counts.device).release()


def test_headline_lists_at_a_large_key_capacity():
    wl = S.headline_workload()
    sc, view = wl.scene, wl.views[0]
    st = renderer.RasterSettings(tile_w=view.tile, tile_h=view.tile)
    dev = torch.device("cuda:0")
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
              for a in (sc.mean, sc.qvec, sc.log_scale, sc.alpha_logit)]
    pr = renderer.project(*params, make_gsx_camera(view.c2w, view.cam), st)
    ntw, nth = st.tiles(view.cam)
    small = bin_and_release(pr, ntw, nth, None)
    large = bin_and_release(pr, ntw, nth, 40 << 20)
    assert small[3] == large[3] > 1_000_000
    for a, b in zip(small[:3], large[:3]):
        np.testing.assert_array_equal(a, b)
    ob = O.bin_gaussians(pr.rect.cpu().numpy(), pr.rect.cpu().numpy()[:, 2:], pr.depth.cpu().numpy(), nth, ntw,
                         stride=4)
    assert ob["K"] == large[3]
    np.testing.assert_array_equal(large[0][:large[3]], ob["ids"])
    np.testing.assert_array_equal(large[1], ob["start"])
    np.testing.assert_array_equal(large[2], ob["end"])


@pytest.mark.parametrize("ntw,nth", [(120, 68), (300, 300)])
def test_large_synthetic_lists_match_oracle(ntw, nth):
    n = LARGE_KEYS + 1_234_567
    rng = np.random.default_rng(ntw)
    tx = rng.integers(0, ntw, n, dtype=np.int32)
    ty = rng.integers(0, nth, n, dtype=np.int32)
    rect = np.stack([tx, ty, tx, ty], axis=1)
    depth = (rng.integers(1, 4000, n).astype(np.float32) * np.float32(0.01)).astype(np.float32)
    counts = np.ones(n, np.int32)
    dev = torch.device("cuda:0")
    # binning reads only the rectangles, depths and counts
    pr = renderer.Projected(None, None, torch.from_numpy(depth).to(dev), None, torch.from_numpy(rect).to(dev),
                            torch.from_numpy(counts).to(dev))
    ids, start, end, K = bin_and_release(pr, ntw, nth, None)
    assert K == n
    ob = O.bin_gaussians(rect, rect[:, 2:], depth, nth, ntw, stride=4)
    assert ob["K"] == n
    np.testing.assert_array_equal(ids[:K], ob["ids"])
    np.testing.assert_array_equal(start, ob["start"])
    np.testing.assert_array_equal(end, ob["end"])
