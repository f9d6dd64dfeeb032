import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        have_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture
def raster_flags_clean():
    """Fails the test if a raster kernel flagged an error (e.g. a bulk-copy
    wait that gave up) while it ran."""
    from gaussian_splatting_3d_gb300 import renderer

    renderer.raster_status(clear=True)
    yield
    flags = renderer.raster_status(clear=True)
    assert flags == 0, f"raster kernels flagged errors: 0x{flags:x}"
