"""bench.py's reference arm (the oracle's CPU step, no device) prints one JSON
line with the keys and units the GPU arm prints, marked impl=reference, on a
bounded sample of the workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    env = dict(os.environ, SPH_REF_BUDGET_S="2")
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "small_dam_break",
                          "--steps", "2", "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True,
                         timeout=600, check=True).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and 1 <= d["steps"] <= 2
    assert d["config"]["particles"] == 32768 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
