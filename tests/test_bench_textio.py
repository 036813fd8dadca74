"""The bench's host-only workload (reference-format text I/O) prints one JSON line
with the contract's keys, and its reader and writer reproduce the reference's
stream loops value for value (runs on CPU, about 10 s)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_textio_bench_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--workload", "textio", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config"):
        assert key in line, key
    assert line["config"]["workload"] == "textio"
    assert line["value"] > 0 and line["steps"] == 1
    assert line["read"]["identical_values"] is True
    assert line["write"]["identical_bytes"] is True
