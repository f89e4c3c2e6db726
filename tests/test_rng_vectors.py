"""Seed streams pinned to published reference outputs (no GPU).

SplitMix64 from state 0 (Vigna's splitmix64.c) and xoshiro256++ from the
state (1, 2, 3, 4) (the reference test of the rand_xoshiro crate, whose
`seed_from_u64` fills the state with four SplitMix64 outputs): the Python
generator (zeno_gb300/rng.py), the oracle's splitmix64 and the library's
host streams (zeno_gb300/csrc/zc_rng.h) all give them. zeno seeds its sampler
and per-shot streams this way (src/exec.rs:213-216, :486), so these pins
carry over to every sampled index the oracle and the library produce.
"""
import os
import shutil
import subprocess

import pytest

from zeno_gb300.rng import Xoshiro256pp, splitmix64

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = 0x9E3779B97F4A7C15
SPLITMIX_FROM_0 = [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F, 0xF88BB8A8724C81EC]
XOSHIRO_FROM_1234 = [41943041, 58720359, 3588806011781223, 3591011842654386, 9228616714210784205,
                     9973669472204895162, 14011001112246962877, 12406186145184390807,
                     15849039046786891736, 10450023813501588000]


def test_python_streams():
    assert [splitmix64((k * GOLDEN) % 2**64) for k in range(4)] == SPLITMIX_FROM_0
    assert Xoshiro256pp(0).s == SPLITMIX_FROM_0
    r = Xoshiro256pp(0)
    r.s = [1, 2, 3, 4]
    assert [r.next_u64() for _ in range(10)] == XOSHIRO_FROM_1234


def test_oracle_splitmix(oracle):
    assert [oracle.lib().zo_splitmix64((k * GOLDEN) % 2**64) for k in range(4)] == SPLITMIX_FROM_0


def test_library_streams(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ is missing")
    exe = str(tmp_path / "rng_harness")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "zeno_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "rng_harness.cpp"), "-o", exe], check=True)
    assert subprocess.run([exe], check=True, capture_output=True, text=True).stdout.strip() == "ok"
