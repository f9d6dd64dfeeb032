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
