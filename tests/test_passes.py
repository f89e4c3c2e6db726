"""Register passes of double-float sweeps, checked on the host (no GPU).

tests/passes_harness.cpp plans random micro-op lists on one tile (2^9
amplitudes, and the double-float kernel's own 2^12) with plan_passes (zeno_gb300/csrc/zc_passes.h, the code the sweep kernel
runs once per job), applies each pass the way the kernel does (the folded CX
block as an affine load map, the fused table diagonal indexed from the
descriptor, rows flipped at the store) and compares with the micro-ops applied
one by one: with and without CX folding, register groups of two and three.
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


def _run_harness(name, tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / name)
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + CSRC, "-I" + inc,
                    os.path.join(ROOT, "tests", name + ".cpp"), "-o", exe], check=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout


def test_passes_apply_the_micro_ops(tmp_path):
    out = _run_harness("passes_harness", tmp_path)
    m = re.match(r"ok worst (\S+) passes (\d+) folded (\d+) fused (\d+) translations (\d+)", out)
    assert m, out
    assert float(m[1]) < 1e-12
    # every feature of the descriptors was exercised
    assert all(int(m[i]) > 1000 for i in range(2, 6)), out

