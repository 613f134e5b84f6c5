"""`bench.py --impl reference` (the reference's CPU estimator on the host
cores) prints one JSON line with the base contract's keys, on a small
workload and a short per-step budget."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "tg64", "--steps", "2",
                        "--warmup", "1", "--ref-seconds", "0.2"], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["unit"] == "particle-steps/s"
    assert out["value"] > 0 and out["steps"] == 2 and out["warmup"] == 1 and out["higher_is_better"] is True
    assert out["config"]["workload"] == "tg64" and out["config"]["N"] == 64 * 64
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == out["value"]
    assert out["e2e"] == {"value": out["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}
