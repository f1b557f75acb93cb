"""bench.py's reference arm runs on the host cores alone: the FP64 oracle port timed through a
persistent pool, with the JSON line the driver reads.  It must not map the engine library
(the arm anchors the comparison, so it may not run any of the product's code).  No GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "12flies_fixed",
           "--steps", "3", "--warmup", "3", "--ref-regions", "3", "--cpu-cores", "2"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["steps"] == 3 and line["warmup"] == 3
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["failed_regions"] == 0
    assert not any("phylocsf_gb300" in lib for lib in line["native_libs_loaded"])
