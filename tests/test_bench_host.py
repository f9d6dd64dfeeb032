"""The measurement contract of bench.py that needs no GPU.

* ``--impl reference`` on the CPU-runnable workload (10k Gaussians, 256x256)
  prints one JSON line with the base keys, ``impl: reference``, a
  ``cpu_baseline`` describing the run and an ``e2e`` with zero copies;
* ``--impl reference-cuda`` prints its ``unavailable`` line and exits 0;
* the roofline's committed ncu figures are found in ``profiles/``;
* the per-launch algorithmic bytes follow the per-unit figures the
  roofline is documented with.
"""
import json
import os
import subprocess
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _run(*args, timeout=600, wall=None):
    t0 = time.perf_counter()
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                       capture_output=True, text=True, timeout=timeout)
    if wall is not None:
        wall.append(time.perf_counter() - t0)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_line_on_the_small_workload():
    pytest.importorskip("torch")
    wall = []
    d = _run("--impl", "reference", "--workload", "small", "--steps", "3", "--warmup", "3", wall=wall)
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["higher_is_better"] is False and d["unit"] == "ms/iter" and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "ms/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("small")
    # a measurement of whole steps, not an extrapolation: the claimed step
    # time over the timed steps fits inside the process's own wall time
    assert d["value"] * 1e-3 * d["steps"] <= wall[0]
    assert cb["stats_ms"]["n"] == 3 and cb["stats_ms"]["p99"] >= cb["stats_ms"]["median"]
    # the same config keys the GPU arm prints (visible Gaussians and keys from the oracle)
    from gaussian_splatting_3d_gb300 import scene as S

    want = bench.workload_config(S.small_workload(), "small", d["config"]["visible"], d["config"]["keys"], 1)
    assert d["config"] == want and d["config"]["keys"] > 0


def test_reference_cuda_arm_is_unavailable():
    d = _run("--impl", "reference-cuda", timeout=120)
    assert d["impl"] == "reference-cuda" and "device assert" in d["unavailable"]


def test_profiled_figures_are_committed():
    t = bench.profiled_traffic("raster_bwd", "headline")
    assert t is not None and t[0] > 0 and t[1].startswith("profiles" + os.sep)
    w = bench.profiled_traffic("raster_bwd", "headline", "warp_inst_per_launch")
    assert w is not None and w[0] > 1e8
    assert bench.profiled_traffic("no_such_kernel", "headline") is None


def test_algorithmic_bytes_per_unit():
    n, K, P, C, T = 1000, 5000, 640 * 480, 4, 1200
    CC = C * C
    assert bench.algorithmic_bytes("raster_fwd", n, K, P, C, T) == K * (28 + 12 * CC) + 12 * P
    assert bench.algorithmic_bytes("raster_bwd", n, K, P, C, T) == (
        K * (28 + 12 * CC) + 24 * P + K * 4 * (3 * CC + 7))
    assert bench.algorithmic_bytes("project", n, K, P, C, T) == n * 96
    assert bench.algorithmic_bytes("project_bwd", n, K, P, C, T) == n * 120
    assert bench.algorithmic_bytes("binning", n, K, P, C, T) == n * 96 + K * 48 + 8 * T
    assert bench.algorithmic_bytes("unknown", n, K, P, C, T) == 0


def test_secondary_workload_failures_are_recorded(monkeypatch):
    """A secondary run that exits non-zero or prints no line leaves its
    reason under its name instead of stopping the headline line."""
    monkeypatch.setattr(bench, "SECONDARY", (("no-such-workload", ["--steps", "1"], 60),))
    out = bench.secondary_workloads()
    rec = out["no-such-workload"]
    assert rec["error"].startswith("exit 2") and rec["args"] == ["--steps", "1"]
