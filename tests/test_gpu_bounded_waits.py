"""Failure detection of the raster's bounded waits, without a GPU fault.

The raster stages SH rows with bulk copies and waits for them on an mbarrier
with a poll limit; on expiry it sets a sticky error bit (read by
gsx_raster_status) instead of hanging or trapping.  The diagnostic entry point
runs the same bounded wait on a barrier phase that cannot complete, so the
limit runs out: the status must report it, and the context must stay usable.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import _lib, renderer, scene as S  # noqa: E402
from gaussian_splatting_3d_gb300._torch import ptr, stream_handle  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports():
    dev = torch.device("cuda:0")
    renderer.raster_status(dev, clear=True)
    polls = torch.zeros(1, dtype=torch.int32, device=dev)
    limit = 4096
    _lib.call("gsx_raster_wait_selftest", limit, ptr(polls), stream_handle(dev))
    torch.cuda.synchronize()
    assert int(polls.item()) == limit
    assert renderer.raster_status(dev, clear=True) & 1
    assert renderer.raster_status(dev, clear=True) == 0  # cleared
    # the context is still usable: a normal render matches the oracle
    wl = S.custom_workload(1500, 64, 48, 3, seed=47)
    sc, view = wl.scene, wl.views[0]
    params = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
              for a in (sc.mean, sc.qvec, sc.log_scale, sc.sh, sc.alpha_logit)]
    img = renderer.rasterize(*params, view.c2w, view.cam, renderer.RasterSettings())
    ref = O.render_view(sc, view)
    assert np.abs(img.cpu().numpy() - ref["image"]).max() <= 2e-6
    assert renderer.raster_status(dev, clear=True) == 0


def test_selftest_limit_is_validated_on_the_host():
    lib = _lib.load()
    assert lib.gsx_raster_wait_selftest(0, ctypes.c_void_p(1 << 40), None) == _lib.GSX_ERR_INVALID_ARG
    assert lib.gsx_raster_wait_selftest((1 << 20) + 1, ctypes.c_void_p(1 << 40), None) == _lib.GSX_ERR_INVALID_ARG


def test_sort_look_back_wait_gives_up_and_reports():
    """A onesweep chunk whose predecessor never publishes stops waiting after
    its poll limit: the pass reports GSX_ERR_TIMEOUT and the device stays
    usable (a binning afterwards is exact)."""
    dev = torch.device("cuda:0")
    lib = _lib.load()
    scratch = torch.empty(lib.gsx_look_back_selftest_bytes(), dtype=torch.uint8, device=dev)
    bits = ctypes.c_uint32(0)
    st = lib.gsx_look_back_selftest(ptr(scratch), scratch.numel(), ctypes.byref(bits), stream_handle(dev))
    assert st == _lib.GSX_ERR_TIMEOUT, lib.gsx_last_error()
    assert bits.value & 1
    wl = S.custom_workload(2000, 96, 64, 1, seed=53)
    ref = O.render_view(wl.scene, wl.views[0])
    pr = ref["proj"]
    t = lambda a, dt=torch.float32: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)  # noqa: E731
    proj = renderer.Projected(t(pr["mean2d"]), t(pr["cov2d"]), t(pr["depth"]), t(pr["alpha"]),
                              t(pr["rect"], torch.int32), t(pr["counts"], torch.int32))
    ids, start, end, K = renderer.bin_gaussians(proj, 6, 4)
    assert K == ref["bins"]["K"]
    np.testing.assert_array_equal(ids.cpu().numpy(), ref["bins"]["ids"])
