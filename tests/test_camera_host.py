"""Host-side camera record: memoisation of make_gsx_camera (CPU only)."""
import numpy as np

from gaussian_splatting_3d_gb300.camera import CameraInfo, frustum_np, look_at_c2w, make_gsx_camera


def _record(g):
    return (list(g.c2w), g.fx, g.fy, g.cx, g.cy, g.width, g.height, list(g.frustum_normals), list(g.frustum_pts))


def test_camera_record_is_memoised_on_the_exact_camera():
    cam = CameraInfo.from_vertical_fov(50.0, 640, 360)
    c2w = look_at_c2w((0.0, -8.0, 1.0))
    a = make_gsx_camera(c2w, cam)
    assert make_gsx_camera(c2w.copy(), cam) is a
    n, p = frustum_np(c2w, cam)
    assert list(a.frustum_normals) == [float(v) for v in n.reshape(-1)]
    assert list(a.frustum_pts) == [float(v) for v in p.reshape(-1)]
    # one ulp in c2w, or a changed CameraInfo, gives a fresh record
    c2 = c2w.copy()
    c2[0, 3] = np.nextafter(c2[0, 3], np.float32(1.0))
    assert make_gsx_camera(c2, cam) is not a
    cam2 = CameraInfo.from_vertical_fov(50.0, 640, 360)
    cam2.downsample(2)
    b = make_gsx_camera(c2w, cam2)
    assert b is not a and (b.width, b.height) == (320, 180)
    assert _record(make_gsx_camera(c2w, cam)) == _record(a)
