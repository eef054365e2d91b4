"""bench.py's reference arm on a small workload: the reference's CPU step (the
library compiled from its own sources where they are staged, else the oracle)
on the host's cores prints one JSON line with the contract's keys, its
all-cores figure and one core's figure."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_its_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--worlds", "8", "--steps", "2",
           "--warmup", "1", "--settle", "3"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, res.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "config", "cpu_baseline", "single_thread", "e2e"):
        assert key in out, key
    assert out["steps"] == 2 and out["unit"] == "body-steps/s" and out["higher_is_better"] is True
    assert out["value"] > 0 and out["single_thread"]["value"] > 0
    assert out["cpu_baseline"]["kind"] in ("reference", "port")
    assert out["cpu_baseline"]["cores"] == out["config"]["processes"] >= 1
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["d2h_bytes_per_step"] == 0
