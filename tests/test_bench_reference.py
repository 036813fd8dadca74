"""The bench's reference arm (`--impl reference`): the reference's CPU implementation of
the path (the FP64 restatement, every host thread) on a bounded sample of the same
workload, printed as one JSON line with the contract's keys and the same `config` as
the repo's arm.  Without its ref_cuda_* legs it needs no GPU; under a multi-rank
launch only rank 0 works and prints.  Runs on CPU in a few seconds."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
CMD = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "cfg1_1MHz", "--steps", "1",
       "--warmup", "1", "--no-ref-cuda", "--cpu-seconds", "1"]


def test_reference_arm_line():
    r = subprocess.run(CMD, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the same workload description as the repo's arm prints for this workload
    sys.path.insert(0, str(ROOT))
    import bench
    from viss_recon_shade_gb300.synth import WORKLOADS
    wl = WORKLOADS["cfg1_1MHz"]
    c = line["config"]
    assert c == bench.workload_config(wl, c["K"], c["J"], c["precision"], 1, "geometric")
    assert c["K"] == wl.snapshots * wl.npairs and c["J"] == wl.J


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    r = subprocess.run(CMD, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
