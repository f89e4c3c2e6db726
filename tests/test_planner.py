"""Host logic of the sweep planner (no GPU).

tests/planner_harness.cpp plans random programs sweep by sweep through the
built library's own plan_sweep / consume_plan — on 11 qubits with small
tiles (ops on outer qubits and carried diagonals occur), and on 15 qubits
with the kernel's own tile shapes (256-byte rows, 7 high qubits) — decodes each
sweep's encoded micro-ops through its tile geometry, applies them in
complex<double> and compares with the program applied directly: identical
in exact mode (ops kept as given), within 1e-11 for the fast f64 lowering,
within 1e-5 for fast f32 (float tables).
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "zeno_gb300", "csrc")


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    return None


def test_planned_sweeps_match_the_program(zc, tmp_path):
    from zeno_gb300 import build

    cxx = shutil.which("g++")
    inc = _cuda_include()
    lib = build.LIB
    if cxx is None or inc is None or not os.path.exists(lib):
        pytest.skip("g++, the CUDA headers or the built library are missing")
    exe = str(tmp_path / "planner_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + CSRC, "-I" + inc,
                    os.path.join(ROOT, "tests", "planner_harness.cpp"), lib,
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    m = re.match(r"ok exact (\S+) fast64 (\S+) fast32 (\S+) sweeps (\d+) carried (\d+)", out)
    assert m, out
    assert float(m[1]) == 0.0
    assert float(m[2]) < 1e-11 and float(m[3]) < 1e-5
    assert int(m[4]) > 100 and int(m[5]) > 0
