"""The serving output arena (admission budget bookkeeping) on the CPU:
random admissions and out-of-order releases against an independent model."""
import os
import subprocess

from conftest import ROOT


def test_arena_properties(tmp_path):
    exe = str(tmp_path / "check_arena")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "mrg8_gb300", "csrc"), "-o", exe,
                    os.path.join(ROOT, "tests", "native", "check_arena.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
    assert int(r.stdout.split()[1]) > 10000
