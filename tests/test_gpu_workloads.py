"""The measurement drivers behind bench.py's `configs` (zeno_gb300/workloads.py),
run at small sizes so that a broken driver shows up here rather than in a
benchmark run; and the arithmetic-peak probe the rooflines divide by."""

import pytest

from zeno_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PEAK = 6800.0


def test_arith_peaks_are_plausible(zc):
    p = zc.arith_peaks()
    assert p["sms"] > 0
    assert p["fp64_fma_per_s"] > 1e10 and p["fp32_fma_per_s"] > 10 * p["fp64_fma_per_s"]


def test_fusion_and_big_state_drivers(zc):
    rows = W.fusion_sweep(PEAK, qubits=16, widths=(1, 3))
    assert [r["fusion"] for r in rows] == [1, 3]
    assert all(r["seconds"] > 0 and r["sweeps"] > 0 and r["pass_GBps"] > 0 for r in rows)
    b = W.big_state(PEAK, qubits=17)
    assert b["seconds"] > 0 and b["launches"] > 0


def test_gate_mix_driver_accuracy_columns(zc):
    out = W.gate_mix_tc(PEAK, tf32_tflops=1000.0, qubits=14)
    names = [r["variant"] for r in out["rows"]]
    assert names[0].startswith("f64 sweeps") and names[1].startswith("f32 sweeps") and len(names) == 5
    f64, f32 = out["rows"][0], out["rows"][1]
    assert f64["max_abs_damp_vs_f64"] < 1e-12 and f64["meets_tvd_1e-6"]
    assert f32["max_abs_damp_vs_f64"] < 1e-5
    assert all(r["tc_blocks"] > 0 for r in out["rows"][2:])


def test_serving_driver_small_stream(zc):
    out = W.serving(PEAK, requests=40, rates=(2000.0,), tvd_samples=3, f64_requests=10)
    r = out["rates"][0]
    assert r["server"]["requests"] == 40 and r["one_per_call"]["requests"] == 40
    assert r["throughput_ratio"] > 0
    assert out["all_f64"]["requests"] == 10
    assert out["f32_vs_f64"]["requests"] == 3 and out["f32_vs_f64"]["max_tvd"] < 1e-4
