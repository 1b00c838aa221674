"""CPU test of the page-locked staging ring's bookkeeping
(natural_number_gb300/csrc/stage_ring.h, used by engine.cpp's Stager) with
host-side fake events: tests/cpp/stage_ring_test.cpp, compiled with g++."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ring_reuses_a_region_only_after_its_copy(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ is not installed")
    exe = str(tmp_path / "stage_ring_test")
    subprocess.check_call(["g++", "-std=c++20", "-O1", "-Wall", "-Werror", "-I",
                           os.path.join(ROOT, "natural_number_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "cpp", "stage_ring_test.cpp"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"
