"""Host logic of the double-float sweep lowering (no GPU).

Fast-mode sweeps of f64 states rewrite each one-qubit gate as diagonal *
real * diagonal and carry the diagonals through CX and SWAP into merged
table ops (zeno_gb300/csrc/zc_lower.cpp). tests/lowering_harness.cpp applies
random programs directly and through the lowered ops on a 7-qubit state in
complex<double>; this test builds it with g++ and requires agreement to
1e-12 on every trial, with the whole-matrix fallback exercised.
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


def test_lowering_matches_direct_application(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "lowering_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + CSRC, "-I" + inc,
                    os.path.join(ROOT, "tests", "lowering_harness.cpp"), os.path.join(CSRC, "zc_lower.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    m = re.match(r"ok worst (\S+) gates (\d+) r1 (\d+) rt (\d+) u1 (\d+) dk (\d+) carried (\d+)", out)
    assert m, out
    worst, gates, r1, rt, u1, dk, carried = float(m[1]), *map(int, m.groups()[1:])
    assert worst < 1e-12
    assert r1 > 0 and rt > 0 and u1 > 0 and dk > 0 and carried > 0
    assert r1 + rt + u1 <= gates
