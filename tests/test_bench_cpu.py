"""bench.py's CPU legs, which need no GPU: the reference arm's JSON line
(--impl reference, the oracle's C^2/2 step timed on bounded samples) and the
cpu_baseline object of the GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "3",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "sphere-steps/s @1M" and d["unit"] == "sphere-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 3 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "sphere-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_cpu_baseline_object():
    b = bench.cpu_baseline(sizes=(512, 1024, 2048), target_n=1_000_000)
    assert b["value"] > 0 and b["unit"] == "sphere-steps/s" and b["cores"] == 1 and b["kind"] == "port"
    assert "extrapolated to N=1000000" in b["sample"]


def test_profile_traffic_is_read_from_the_committed_summary():
    t = bench.profile_traffic("k_step_single_1M.md")
    # a launch's DRAM bytes (read + write) of one capture: tens of MB
    assert t is not None and 10e6 < t < 500e6
    assert bench.profile_traffic("no_such_file.md") is None
