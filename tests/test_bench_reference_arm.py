"""bench.py's reference arm (the reference's own solver compiled on the host
where its sources were staged, else the oracle port) prints one contract line
on the host alone, reporting the steps and warm-up it actually ran: the
Gauss-Seidel steps and FLIP at the reference mains' 128 x 128 with the default
step counts, and a small stratified sample of the batched workload."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _line(*extra):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *extra],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def _check(line, steps, warmup, step):
    from oracle import oracle as O
    assert line["impl"] == "reference" and line["metric"] == "cell-steps/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["steps"] == steps and line["warmup"] == warmup
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == ("reference" if O.ref_available(step) else "port")
    assert cb["value"] == line["value"] and cb["steps"] == steps and cb["warmup"] == warmup
    assert abs(line["ms_per_step"] - 1e3 * cb["seconds"] / cb["steps"]) < 1e-6
    return cb


@pytest.mark.parametrize("workload,step", [("gs", 1), ("flip", 8)])
def test_reference_arm_line_default_steps(workload, step):
    cb = _check(_line("--workload", workload), 5, 3, step)
    assert cb["cores"] == 1


def test_reference_arm_batch_sample():
    cb = _check(_line("--workload", "batch", "--steps", "2", "--warmup", "1", "--cpu-sample", "2",
                      "--cpu-procs", "2"), 2, 1, 4)
    assert cb["cores"] == 2 and "2 of the 512 batch scenes" in cb["sample"]
