"""bench.py's reference arm (the reference's CPU algorithm through the oracle)
prints one contract line on the host alone, for the workloads small enough to
run in the CPU suite (the Gauss-Seidel steps and FLIP at the reference mains'
128 x 128)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload", ["gs", "flip"])
def test_reference_arm_line(workload):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        workload, "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=300,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "cell-steps/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == 2 and line["warmup"] == 3
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 1 and cb["value"] == line["value"]
    assert abs(line["ms_per_step"] - 1e3 * cb["seconds"] / cb["steps"]) < 1e-6
