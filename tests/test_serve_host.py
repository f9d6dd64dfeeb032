"""Host-side logic of the render server (no GPU): batch selection under the
memory budget, the binning status block decoder, and the serving workload
generator."""
import ctypes
from types import SimpleNamespace

import numpy as np
import pytest

from gaussian_splatting_3d_gb300 import _lib
from gaussian_splatting_3d_gb300.serve import poisson_requests, select_batch


def reqs(*orders):
    return [SimpleNamespace(rid=i, C=c) for i, c in enumerate(orders)]


def by_count(unit):
    return lambda batch: unit * len(batch)


def test_select_takes_oldest_first_up_to_max_views():
    w = reqs(4, 4, 4, 4, 4)
    assert select_batch(w, lambda r: r.C, 3, 10**9, by_count(1)) == [0, 1, 2]


def test_select_groups_by_sh_order_of_the_oldest():
    w = reqs(1, 4, 1, 4, 1)
    assert select_batch(w, lambda r: r.C, 8, 10**9, by_count(1)) == [0, 2, 4]


def test_select_stops_at_the_budget_without_overtaking():
    w = reqs(4, 4, 4, 4)
    sizes = {0: 10, 1: 50, 2: 5, 3: 5}
    f = lambda batch: sum(sizes[r.rid] for r in batch)  # noqa: E731
    # request 1 does not fit: 2 and 3 would, but they must not overtake it
    assert select_batch(w, lambda r: r.C, 8, 40, f) == [0]
    assert select_batch(w, lambda r: r.C, 8, 5, f) == []
    assert select_batch([], lambda r: r.C, 8, 5, f) == []


def _decode(total, err, cap):
    lib = _lib.load()
    block = (ctypes.c_uint64 * 2)(total, err)
    k = ctypes.c_int64(-1)
    st = lib.gsx_binning_status_decode(ctypes.addressof(block), cap, 4, 4, ctypes.byref(k))
    return st, k.value


def test_status_block_decoder():
    assert _decode(100, 0, 100) == (_lib.GSX_OK, 100)
    assert _decode(101, 0, 100) == (_lib.GSX_ERR_CAPACITY, 101)
    assert _decode(5, 1, 100)[0] == _lib.GSX_ERR_TIMEOUT
    assert _decode(5, 2, 100)[0] == _lib.GSX_ERR_MISMATCH
    assert _decode(5, 4, 100)[0] == _lib.GSX_ERR_INVALID_ARG
    # the upper half of the second word is the key count used, not error bits
    assert _decode(7, 7 << 32, 100) == (_lib.GSX_OK, 7)
    lib = _lib.load()
    assert lib.gsx_binning_status_decode(None, 1, 1, 1, None) == _lib.GSX_ERR_INVALID_ARG


def test_poisson_stream_rate_and_mix():
    arr = poisson_requests(8, rate=2000.0, duration=2.0, seed=0)
    assert abs(len(arr) - 4000) < 4 * np.sqrt(4000)
    t = np.array([a[0] for a in arr])
    assert np.all(np.diff(t) > 0) and t[-1] < 2.0
    scenes = np.bincount([a[1] for a in arr], minlength=8)
    assert scenes.min() > 350
    sizes = {(a[3].w, a[3].h) for a in arr}
    assert sizes == {(512, 512), (1280, 720), (1920, 1080)}
    radii = np.array([np.linalg.norm(a[2][:, 3]) for a in arr])
    assert radii.min() >= 5.0 - 1e-4 and radii.max() <= 10.0 + 1e-4
    again = poisson_requests(8, rate=2000.0, duration=2.0, seed=0)
    assert [a[0] for a in again] == [a[0] for a in arr]


if __name__ == "__main__":
    pytest.main([__file__])
