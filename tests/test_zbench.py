"""`zeno bench` on the GPU (zeno_gb300/zbench.py): zeno's schema-v1 JSON
shape, as tests/cli.rs:173-228 checks it, plus the GPU's pass GB/s."""

import pytest


def test_sizes_over_the_budget_are_skipped(zc, monkeypatch):
    """tests/cli.rs:212-228: pretend 1 MiB of device memory; 26 qubits are
    skipped with the budget in the reason (no device work is needed)."""
    from zeno_gb300 import zbench

    monkeypatch.setenv("ZENO_MEM_BYTES", str(1 << 20))
    v = zbench.bench(zbench.parse(["--qubits", "26,30", "--depth", "2"]))
    assert v["schema_version"] == 1 and v["depth"] == 2 and v["seed"] == 7
    assert [r["skipped"] for r in v["results"]] == [True, True]
    assert "budget" in v["results"][0]["reason"]


@pytest.mark.gpu
def test_bench_json_small_sweep(zc):
    """tests/cli.rs:173-192 and :194-210."""
    from zeno_gb300 import zbench

    v = zbench.bench(zbench.parse(["--qubits", "4,5,20", "--depth", "3", "--compare-fusion"]))
    assert v["schema_version"] == 1 and v["depth"] == 3 and v["seed"] == 7 and v["fusion"] == 1
    assert [r["qubits"] for r in v["results"]] == [4, 5, 20]
    for r in v["results"]:
        assert r["skipped"] is False
        assert r["input_gates"] > 0 and r["output_ops"] > 0
        assert r["sim_time_ms"] >= 0 and r["amp_updates_per_s"] > 0
        assert r["speedup"] > 0 and r["nofusion_time_ms"] >= 0
        assert r["backend"] == "cuda-f64" and r["passes"] > 0 and r["pass_GBps"] > 0
    assert v["notices"] == []
