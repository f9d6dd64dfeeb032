"""The allocation-free binning entry point gives the same lists as the
workspace one.

gsx_tile_culling_aabb_start_end_noalloc serves callers that cannot allocate
device memory (a plugin inside another program's fixed memory budget, a
real-time loop that must not enter the allocator): it borrows a 64 MiB array
in the library's static device memory instead of taking a workspace.  This
test calls both entry points through the C ABI on the same inputs, twice in a
row with different scenes (so leftovers of the first call in the shared
array would show), and requires identical gaussian_ids / start / end -- the
exact-match tolerance every binning test uses -- and the same lists from the
CPU oracle's restatement of the reference binning.  It lives in its own file that
pytest collects last, and passes both alone and after the other tests.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import _lib, scene as S  # noqa: E402
from gaussian_splatting_3d_gb300.camera import frustum_np  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def _rects(seed, n, w, h, sh_degree):
    wl = S.custom_workload(n, w, h, sh_degree, seed=seed)
    sc, view = wl.scene, wl.views[0]
    cam = view.cam
    normals, pts = frustum_np(view.c2w, cam)
    ocam = O.make_camera(view.c2w, cam.fx, cam.fy, cam.cx, cam.cy, cam.w, cam.h, normals, pts)
    pr = O.project(sc.mean, sc.qvec, sc.log_scale, sc.alpha_logit, ocam, 1.0, 6.0, 16, 16)
    m = pr["mask"]
    tl = np.ascontiguousarray(pr["rect"][m][:, :2])
    br = np.ascontiguousarray(pr["rect"][m][:, 2:])
    depth = np.ascontiguousarray(pr["depth"][m])
    K = int(np.prod(br - tl + 1, axis=1).sum())
    return tl, br, depth, K, (cam.w + 15) // 16, (cam.h + 15) // 16


def _bin(entry, tl, br, depth, K, ntw, nth, with_workspace):
    dev = torch.device("cuda:0")
    lib = _lib.load()
    n = tl.shape[0]
    t_tl = torch.from_numpy(tl).to(dev)
    t_br = torch.from_numpy(br).to(dev)
    t_depth = torch.from_numpy(depth).to(dev)
    ids = torch.full((K,), -7, dtype=torch.int32, device=dev)
    start = torch.full((ntw * nth,), -7, dtype=torch.int32, device=dev)
    end = torch.full((ntw * nth,), -7, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    if with_workspace:
        ws_bytes = lib.gsx_binning_workspace_bytes(n, K, ntw * nth)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
        st = getattr(lib, entry)(n, K, t_tl.data_ptr(), t_br.data_ptr(), t_depth.data_ptr(), nth, ntw,
                                 ids.data_ptr(), start.data_ptr(), end.data_ptr(), ws.data_ptr(), ws_bytes,
                                 stream)
    else:
        st = getattr(lib, entry)(n, K, t_tl.data_ptr(), t_br.data_ptr(), t_depth.data_ptr(), nth, ntw,
                                 ids.data_ptr(), start.data_ptr(), end.data_ptr(), stream)
    _lib.check(st, entry)
    assert lib.gsx_last_error() == b""  # a successful call leaves no earlier message behind
    torch.cuda.synchronize()
    return ids.cpu().numpy(), start.cpu().numpy(), end.cpu().numpy()


def test_noalloc_binning_matches_workspace_binning_on_consecutive_calls():
    cases = [_rects(3, 6000, 160, 120, 2), _rects(4, 2500, 96, 64, 0)]
    for tl, br, depth, K, ntw, nth in cases:
        ref = _bin("gsx_tile_culling_aabb_start_end", tl, br, depth, K, ntw, nth, True)
        got = _bin("gsx_tile_culling_aabb_start_end_noalloc", tl, br, depth, K, ntw, nth, False)
        for a, b in zip(got, ref):
            np.testing.assert_array_equal(a, b)
        orc = O.bin_gaussians(tl, br, depth, nth, ntw)
        assert orc["K"] == K
        np.testing.assert_array_equal(got[0], orc["ids"][:K])
        np.testing.assert_array_equal(got[1], orc["start"])
        np.testing.assert_array_equal(got[2], orc["end"])


def test_noalloc_rejects_inputs_beyond_its_scratch():
    lib = _lib.load()
    n, K = 3_000_000, 3_000_000  # about 96 MB of scratch: more than the static array
    st = lib.gsx_tile_culling_aabb_start_end_noalloc(n, K, ctypes.c_void_p(16), ctypes.c_void_p(16),
                                                    ctypes.c_void_p(16), 68, 120, ctypes.c_void_p(16),
                                                    ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert st == _lib.GSX_ERR_CAPACITY
    assert b"static" in lib.gsx_last_error()
