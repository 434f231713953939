"""bench.py's workloads and its reference arm's JSON line (CPU only)."""

from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "tests" / "golden"))
import configs  # noqa: E402

import bench  # noqa: E402


@pytest.mark.parametrize("name,workload", [("bench_fan512", bench.WORKLOAD),
                                           ("bench_radon256", bench.RADON_WORKLOAD)])
def test_bench_workloads_match_fixture_table(name, workload):
    """The bench's geometries are the fixture table's entries that the GPU parity
    tests use (Radon: 363 detectors spanning the image diagonal, 2 sqrt 2)."""
    want = configs.configs()[name]
    assert workload.keys() == want.keys()
    for k in want:
        if isinstance(want[k], str):
            assert workload[k] == want[k], k
        else:
            assert np.allclose(workload[k], want[k], rtol=1e-15, atol=0), k


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps",
                          "1", "--warmup", "3"], capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["warmup"] >= 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert "workload" in d["config"]
