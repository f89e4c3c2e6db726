"""The sampler's host half against the oracle (no GPU).

tests/sampler_harness.cpp routes random states' chunk masses through the
built library's sample_route (serial prefix, serial draws scaled by the
total, ascending sort, routing of draws to chunks), rescans the touched
chunks the way the device's second pass does, and requires the oracle's
sampled indices (src/sample.rs:29-111) at the same seed: f64 and f32 states,
dense, with zero-probability stretches, and nearly empty; 0 to 4096 shots.
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "zeno_gb300", "csrc")


def test_sample_route_matches_the_oracle(zc, oracle, tmp_path):
    from zeno_gb300 import build

    cxx = shutil.which("g++")
    inc = None
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            inc = os.path.join(base, "include")
    lib, olib = build.LIB, oracle.LIB_PATH
    if cxx is None or inc is None or not os.path.exists(lib) or not os.path.exists(olib):
        pytest.skip("g++, the CUDA headers, the built library or the oracle are missing")
    exe = str(tmp_path / "sampler_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + CSRC, "-I" + os.path.join(ROOT, "oracle"),
                    "-I" + inc, os.path.join(ROOT, "tests", "sampler_harness.cpp"), lib, olib,
                    "-Wl,-rpath," + os.path.dirname(lib), "-Wl,-rpath," + os.path.dirname(olib), "-o", exe],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    m = re.match(r"ok cases (\d+) draws (\d+) touched (\d+) leftovers (\d+)", out)
    assert m, out
    assert int(m[1]) == 192 and int(m[2]) > 100000 and int(m[3]) > 144
