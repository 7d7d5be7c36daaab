"""bench.py's contract pieces that run without a GPU: the reference arm's JSON
line (the CPU oracle timed on the host), the byte model of the step floor,
and the readers of the committed ncu summaries the roofline quotes."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402
from natrix_gb300 import workloads as wl  # noqa: E402


def test_reference_arm_line():
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--workload", "small", "--steps", "2", "--warmup", "1"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "cell-updates/s" and line["unit"] == "cell-updates/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1 and line["n_gpus"] == 1
    # the same config dict as the GPU arm's line for this workload
    assert line["config"] == bench.workload_config(wl.SMALL_256, {"parallelism": "replicas1"})
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["kind"] in ("reference", "port")
    assert cpu["cores"] >= 1 and cpu["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_step_floor_of_the_large_workload():
    # forcing 24, advection 17, density advection 17, divergence 18, vorticity
    # 20, ten 8-sweep chunks of 13, the gradient fused into the last one (16)
    assert bench.step_floor_bytes_per_cell(wl.LARGE_2048, 10, 1.0) == 242
    # the gradient subtraction in a launch of its own instead
    assert bench.step_floor_bytes_per_cell(wl.LARGE_2048, 10, 0.0) == 247


def test_committed_profiles_parse():
    chain = "jacobi_chain_2048x2048.txt"
    assert bench.load_traffic(chain) == pytest.approx(94.367e6)
    assert bench.load_instructions(chain) == pytest.approx(141.18e6, rel=1e-3)
    per_chunk = "jacobi_rt_2048x2048.txt"
    assert bench.load_traffic(per_chunk) == pytest.approx(37.921e6)
    assert bench.load_instructions(per_chunk) == pytest.approx(13.17e6, rel=1e-3)
    assert bench.load_traffic("no_such_profile.txt") is None
    assert bench.load_instructions("no_such_profile.txt") is None
