"""The bench's line for the repo's arm on a small configuration (10 MHz, 458,752 x 49,152):
the contract's keys, an end-to-end figure with host copies, a roofline fraction of the
measured SFU peak, sampled clocks and the count of the repo's own kernel launches."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_bench_line_cfg4():
    cmd = [sys.executable, str(ROOT / "bench.py"), "--workload", "cfg4_10MHz", "--steps", "2", "--warmup", "3",
           "--no-cpu-baseline", "--no-plain", "--no-stage1", "--no-batch", "--no-largest", "--no-ref-cuda"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "clocks", "gpu_launches"):
        assert key in line, key
    assert line["config"]["workload"] == "cfg4_10MHz" and line["steps"] == 2 and line["warmup"] == 3
    assert line["value"] > 100  # Gterms/s; the repo's kernels, not a fallback
    e2e = line["e2e"]
    assert e2e["value"] > 0 and e2e["h2d_bytes_per_step"] > 0 and e2e["d2h_bytes_per_step"] > 0
    rf = line["roofline"]
    assert rf["bound"] == "sfu" and 0.3 < rf["frac"] < 1.5 and rf["peak"] > 0
    assert line["gpu_launches"] >= 2 * line["steps"]
    assert line["clocks"]["samples"] >= 1
