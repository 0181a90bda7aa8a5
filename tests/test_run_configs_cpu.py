"""The CPU leg of tests/run_configs.py (the CPU restatement timings) runs and
reports one row per chi and element type."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpu_timing_config_runs():
    cmd = [sys.executable, os.path.join(ROOT, "tests", "run_configs.py"), "cpu1", "--cpu-reps", "1",
           "--c2-chis", "4", "8"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300, check=True)
    out = json.loads(res.stdout.strip().splitlines()[-1])
    assert out["config"] == "cpu1"
    rows = {(r["chi"], r["dtype"]): r for r in out["rows"]}
    assert set(rows) == {(4, "c128"), (4, "c64"), (8, "c128"), (8, "c64")}
    assert all(r["updates_per_s"] > 0 for r in rows.values())
