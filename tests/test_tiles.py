"""How batches cut instances into tiles (mrg8_gb300/csrc/mrg8g_tiles.h, shared
by the batch kernel and the host planner): exact coverage, head and body
alignment, largest-first order, and listed and derived tilings agreeing
(tests/native/check_tiles.cpp).  No GPU needed."""
import os
import subprocess

from conftest import ROOT


def test_tiles_cover_every_instance_and_both_tilings_agree(tmp_path):
    from mrg8_gb300 import build
    exe = str(tmp_path / "check_tiles")
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(build.nvcc()))), "include")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "mrg8_gb300", "csrc"), "-I" + cuda_inc,
                    "-o", exe, os.path.join(ROOT, "tests", "native", "check_tiles.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
