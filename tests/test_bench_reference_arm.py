"""bench.py's reference arm (--impl reference): the CPU restatement of the
reference timed on the host's cores prints one JSON line with the keys the
comparison reads, for the headline and for the other workloads."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("extra", [
    ["--nx", "16"],
    ["--workload", "sod1d", "--nx", "100"],
    ["--workload", "kh2d_selfgrav", "--nx", "16"],
    ["--workload", "kh2d_solver", "--riemann", "AIRS", "--nx", "16"],
    ["--workload", "kh2d_solver", "--riemann", "HLLC", "--runner", "Godunov", "--nx", "16"],
])
def test_reference_arm_line(extra):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3"] + extra,
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "active-face updates/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 2 and line["warmup"] == 3
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["config"]["cells"] > 0
