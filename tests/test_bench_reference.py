"""bench.py's reference arm (the FP32 oracle on the host cores) on a tiny grid,
both physics: it runs without a GPU, prints one JSON line with the fields the
benchmark contract asks for, and keeps the workload's configuration."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("physics", ["psv", "sh"])
def test_reference_arm_runs_on_the_host(physics):
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--physics", physics, "--grid", "48", "--nt", "8",
           "--ref-sample", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == line["metric"]
    assert line["config"]["physics"] == physics and line["config"]["grid"] == [48, 48]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
