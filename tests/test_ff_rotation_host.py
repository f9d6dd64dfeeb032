"""The projection backward's rotation in float-float, checked on the CPU: the
same header (csrc/ff_rot.cuh) built for the host by nvcc with contraction
off, against R(q / |q|) and M = R diag(s) in double precision, for 200,000
seeded quaternions of several magnitudes.  R's float part must be within
2^-23 of the exact entry (it is the rounding of a value exact to ~2^-44)
and M must be the correctly rounded product in all but a handful of
near-tie cases (at most half an ulp off in any case)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def ff_check(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("ff") / "ff_rot_check"
    cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-I",
           str(ROOT / "gaussian_splatting_3d_gb300" / "csrc"), "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "host_src" / "ff_rot_check.cu"), "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, timeout=300)
    r = subprocess.run([str(out)], check=True, capture_output=True, text=True, timeout=120)
    max_r, max_m_ulp, mism, n = r.stdout.split()
    return float(max_r), float(max_m_ulp), int(mism), int(n)


def test_rotation_entries_are_rounded_exact_values(ff_check):
    max_r, _, _, _ = ff_check
    assert max_r <= 2.0 ** -23


def test_scaled_axes_are_correctly_rounded(ff_check):
    _, max_m_ulp, mism, n = ff_check
    assert max_m_ulp <= 0.5 + 1e-6
    assert mism <= n * 9 // 10000  # near-ties only
