"""resolve_precision (src/exec.rs:261-304) in zc_run, against the HBM budget.

An explicit precision must fit the budget (mem::plan, src/mem.rs:114-131:
Error::Memory, ZC_ERR_MEMORY here); automatic precision takes f64 when it
fits, else f32 with zeno's `auto-precision` notice, and refuses when f32
does not fit either. ZENO_MEM_BYTES pretends the device is smaller, as
zeno's own tests do with a machine's RAM (tests/cli.rs:126-153).
"""

import pytest

from zeno_gb300 import circuit as C


def _prog(n, measure=True):
    return C.matching_circuit(n, 2, 3, measure=measure).to_program()


def test_refusal_when_nothing_fits(zc, monkeypatch):
    """20 qubits need 8 MiB at f32; a 1 MiB device (0.75 MiB budget) fits
    neither precision: refused before any device work."""
    monkeypatch.setenv("ZENO_MEM_BYTES", str(1 << 20))
    p = _prog(20)
    with pytest.raises(zc.ZenoCudaError) as e:
        zc.run(p, shots=16, precision=0)
    assert e.value.code == zc.ZC_ERR_MEMORY
    assert "state vector for 20 qubits at f32 needs" in str(e.value)
    with pytest.raises(zc.ZenoCudaError) as e:
        zc.run(p, shots=16, precision=64)
    assert e.value.code == zc.ZC_ERR_MEMORY and "at f64" in str(e.value)


@pytest.mark.gpu
def test_auto_precision_falls_back_to_f32_with_notice(zc, oracle, monkeypatch):
    """A 16 MiB device gives a 12 MiB budget: 20 qubits need 16 MiB at f64,
    8 MiB at f32."""
    monkeypatch.setenv("ZENO_MEM_BYTES", str(16 << 20))
    p = _prog(20)
    r = zc.run(p, shots=2000, seed=5, precision=0)
    assert r.precision == 32 and r.backend == "cuda-f32"
    assert r.notices == ["auto-precision: 20 qubits exceed the f64 budget, using f32 (8 B/amplitude)"]
    want, _, _, _ = oracle.run(p, prec=32, shots=2000, seed=5)
    assert r.counts == want
    with pytest.raises(zc.ZenoCudaError) as e:  # an explicit f64 must fit
        zc.run(p, shots=16, precision=64)
    assert e.value.code == zc.ZC_ERR_MEMORY
    monkeypatch.delenv("ZENO_MEM_BYTES")
    r = zc.run(p, shots=16, seed=5, precision=0)
    assert r.precision == 64 and r.notices == []


@pytest.mark.gpu
def test_run_notices(zc):
    """The other notices zeno's executor pushes (src/exec.rs:374, :429-435)."""
    r = zc.run(_prog(6, measure=False), shots=10, precision=64)
    assert r.notices == ["circuit has no measurements: counts are empty (use --statevector to inspect the state)"]
    assert r.counts == {}
    noise = zc.NoiseModel(depolarizing_1q=1e-3)
    r = zc.run(_prog(6), shots=64, precision=32, noise=noise)
    assert r.notices == ["noise: trajectory sampling — per-shot execution, fusion disabled"]
