"""Host logic of the serving engine (no GPU).

tests/pool_harness.cpp drives the pool allocator the server admits requests
with (zeno_gb300/csrc/zc_pool.h) through random request streams under the
server's admission rule (FIFO; admitted while a slot is free and the state
fits): every allocation is the first fit, the free list stays sorted, merged
and disjoint from the live states, free and live blocks cover the pool, every
request finishes, and an empty pool is one block again.
"""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "zeno_gb300", "csrc")


def test_pool_allocator_and_admission(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ is missing")
    exe = str(tmp_path / "pool_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + CSRC,
                    os.path.join(ROOT, "tests", "pool_harness.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    m = re.match(r"ok allocs (\d+) waits (\d+) finished (\d+) empty_pools_whole (\d+)", out)
    assert m, out
    assert int(m[1]) == int(m[3]) > 10000  # every admitted request finished
    assert int(m[2]) > 1000                # the pool was full often enough to make requests wait
    assert int(m[4]) == 400
