"""The trajectory engine's generator on the host (no GPU).

tests/philox_harness.cpp checks Philox4x32-10 (zeno_gb300/csrc/zc_philox.h,
the code the trajectory kernel draws with) against the known-answer vectors
published with the Random123 library, the stream's counter layout (block i of
trajectory t is counter (i, t), key = seed), and the f64 and integer-range
conversions (bounds, mean, uniform bins at 6 sigma).
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "zeno_gb300", "csrc")


def test_philox_known_answers_and_conversions(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ is missing")
    exe = str(tmp_path / "philox_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + CSRC,
                    os.path.join(ROOT, "tests", "philox_harness.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    assert out.startswith("ok kats 3"), out
