"""The JSON line contract of bench.py, checked on the CPU through the reference
arm (the reference's CPU path on a small workload): one line, the metric and
unit of the headline, a config with the same keys and values as the GPU arm's
for the same workload, both CPU baselines with their core counts, and the e2e
object."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_line(tmp_path):
    n = 1 << 20
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                        "--warmup", "1", "--n", str(n), "--skip-ref-gpu"],
                       capture_output=True, text=True, timeout=600, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["config"] == bench.workload_config(n, 1)
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 1
    cpu = line["cpu_baseline"]
    assert cpu["cores"] >= 1 and cpu["kind"] in ("port", "reference") and cpu["value"] == line["value"]
    assert cpu["scalar_original"]["cores"] == 1 and cpu["scalar_original"]["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["ref_gpu"] is None
