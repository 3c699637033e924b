"""The benchmark's reference arm runs on the CPU: one JSON line with the
metric, the CPU baseline and an end-to-end block that moves no bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-seconds", "2"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "assembled elements/s (tangent+residual)" and line["unit"] == "elements/s"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["steps"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert abs(cb["per_core"] * cb["cores"] - cb["value"]) <= 1e-12 * cb["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "elements/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
