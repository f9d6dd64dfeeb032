"""The raster's exponential on the GPU, bit for bit.

gsx_expf (the projection's form and the CPU oracle's) against the oracle's
orc_expf on a sample of exponents; the raster's branch-free form for
exponents <= 0 and its paired float2 form against gsx_expf on every 53rd
non-positive float down to -87.5, on uniform draws, and on the edges: 0,
-0, the -87 cut and its neighbours, denormals, -inf and NaN.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from gaussian_splatting_3d_gb300 import _lib  # noqa: E402
from gaussian_splatting_3d_gb300._torch import ptr  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


def gpu_exp(x: np.ndarray, variant: int) -> np.ndarray:
    dev = torch.device("cuda:0")
    xd = torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(dev)
    out = torch.full_like(xd, 7.0)
    _lib.check(_lib.load().gsx_exp_selftest(ptr(xd), xd.numel(), ptr(out), variant, None), "gsx_exp_selftest")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def edge_values() -> np.ndarray:
    f = np.float32
    vals = [0.0, -0.0, -87.0, np.nextafter(f(-87.0), f(0.0)), np.nextafter(f(-87.0), f(-1e9)), -87.5, -88.0,
            -1e-45, -1e-40, -1e-38, -np.inf, np.nan, -0.5, -1.0, -np.log(2.0), -10 * np.log(2.0), -86.99]
    return np.array(vals, np.float32)


def nonpositive_inputs() -> np.ndarray:
    # every 53rd bit pattern from -0 down to -87.5, plus uniform draws
    top = np.float32(-87.5).view(np.uint32)
    bits = np.arange(np.uint32(0x80000000), top, 53, dtype=np.uint64).astype(np.uint32)
    sweep = bits.view(np.float32)
    rng = np.random.default_rng(3)
    draws = -rng.random(1 << 20, dtype=np.float32) * np.float32(90.0)
    return np.concatenate([edge_values(), sweep, draws]).astype(np.float32)


def same_bits(a: np.ndarray, b: np.ndarray) -> bool:
    both_nan = np.isnan(a) & np.isnan(b)
    return bool(np.all(both_nan | (a.view(np.uint32) == b.view(np.uint32))))


def test_gsx_expf_matches_the_oracle():
    rng = np.random.default_rng(4)
    xs = np.concatenate([edge_values(), rng.uniform(-100, 100, 20000).astype(np.float32)])
    got = gpu_exp(xs, 0)
    want = np.array([O.expf(x) for x in xs], np.float32)
    assert same_bits(got, want)


@pytest.mark.parametrize("variant", [1, 2])
def test_raster_forms_equal_gsx_expf(variant):
    xs = nonpositive_inputs()
    assert xs.size > 20_000_000
    assert same_bits(gpu_exp(xs, variant), gpu_exp(xs, 0))


def test_paired_form_with_an_odd_count():
    xs = edge_values()[:5]
    assert same_bits(gpu_exp(xs, 2), gpu_exp(xs, 0))
