"""End-to-end parity: compile + run on the CUDA backend against the oracle's
run_program on the same programs and seeds (counts identical; state
vectors bit-identical in exact mode), plus size-independent properties at
full sizes (inverse round trips, norm)."""

import math

import numpy as np
import pytest

import refmats
from helpers import bits_equal, program_from_json
from zeno_gb300 import circuit as C

pytestmark = pytest.mark.gpu


def test_examples_match_oracle(zc, oracle, examples):
    """Same counts as the oracle at the same seed. Dynamic programs take the
    per-shot replay here (ZC_FLAG_PER_SHOT): at f32 they would otherwise run
    as batched trajectories, which agree in distribution only
    (tests/test_gpu_dynamic.py)."""
    for name, d in examples.items():
        p = program_from_json(d)
        dynamic = zc.compile(p, 1).dynamic
        for prec in (64, 32):
            flags = zc.FLAG_PER_SHOT if dynamic else zc.FLAG_EXACT
            mine = zc.run(p, shots=4000, seed=11, precision=prec, fusion=1, flags=flags)
            ref, _, _, _ = oracle.run(p, prec=prec, shots=4000, seed=11, fusion=1)
            assert mine.counts == ref, (name, prec)
        exp = d["expected"]
        if exp["kind"] == "exact":
            assert mine.counts == {exp["keys"][0]: 4000}


@pytest.mark.parametrize("prec", (64, 32))
def test_matching_circuit_20q_counts_and_state(zc, oracle, prec):
    """20-qubit depth-12 u3 + perfect-matching CX, 1024 shots."""
    p = C.matching_circuit(20, 12, 7).to_program()
    mine = zc.run(p, shots=1024, seed=7, precision=prec, statevector=True)
    ref, _, sv, _ = oracle.run(p, prec=prec, shots=1024, seed=7, statevector=True)
    assert bits_equal(mine.statevector, sv)
    assert mine.counts == ref


@pytest.mark.parametrize("fusion", range(0, 7))
def test_random_circuit_every_fusion(zc, oracle, fusion):
    for n in (3, 7, 11):
        p = C.random_circuit(n, 20, 1000 + n).to_program()
        mine = zc.run(p, shots=0, fusion=fusion, precision=64, statevector=True)
        _, _, sv, _ = oracle.run(p, prec=64, shots=0, fusion=fusion, statevector=True)
        assert bits_equal(mine.statevector, sv), (n, fusion)


def test_qft_with_swaps(zc, oracle):
    c, x = C.qft_circuit(12, 3)
    p = c.to_program()
    mine = zc.run(p, shots=8192, seed=1, precision=64, statevector=True)
    ref, _, sv, _ = oracle.run(p, prec=64, shots=8192, seed=1, statevector=True)
    assert np.abs(mine.statevector - sv).max() == 0.0
    assert mine.counts == ref
    dim = 1 << 12
    want = np.exp(2j * math.pi * x * np.arange(dim) / dim) / math.sqrt(dim)
    assert np.abs(mine.statevector - want).max() < 1e-12


def test_dynamic_teleport_and_noise_bit_exact(zc, oracle, examples):
    p = program_from_json(examples["teleport"])
    assert zc.run(p, shots=500, seed=4).counts == oracle.run(p, shots=500, seed=4)[0]
    noise = zc.NoiseModel(depolarizing_1q=0.01, depolarizing_2q=0.05, amplitude_damping=0.02,
                          bit_flip=0.01, phase_flip=0.01, readout_flip_0to1=0.03, readout_flip_1to0=0.02)
    c = C.matching_circuit(5, 3, 21)
    mine = zc.run(c.to_program(), shots=200, seed=8, noise=noise, precision=64)
    ref = oracle.run(c.to_program(), prec=64, shots=200, seed=8, noise=noise)[0]
    assert mine.counts == ref


def test_mixed_circuit_f32_vs_f64(zc):
    p = C.mixed_circuit(14, 20, 5).to_program()
    a = zc.run(p, shots=0, precision=64, statevector=True, fusion=5).statevector
    b = zc.run(p, shots=0, precision=32, statevector=True, fusion=5).statevector
    assert np.abs(a - b).max() < 2e-4


@pytest.mark.parametrize("n,prec,depth,fast", [(26, 64, 3, False), (28, 32, 3, False), (30, 64, 40, True)])
def test_full_size_inverse_round_trip(zc, n, prec, depth, fast):
    """U followed by U^dagger returns |0...0> (size-independent property);
    the last case is the headline workload itself (30 qubits, depth 40, f64,
    double-float arithmetic)."""
    c = C.matching_circuit(n, depth, 99, measure=False)
    inv = C.Circuit(n)
    for ins in reversed(c.instrs):
        if ins.name == "u3":
            t, ph, la = ins.params
            inv.u(ins.qubits[0], -t, -la, -ph)
        else:
            inv.gate(ins.name, ins.qubits, ins.params)
    g = zc.CudaBackend(n, prec, zc.FLAG_FAST if fast else zc.FLAG_EXACT)
    for prog in (c, inv):
        for op in zc.compile(prog.to_program(), 1).ops:
            if op.kind == zc.OP_UNITARY:
                g.apply_unitary(op.qubits, op.data)
            elif op.kind == zc.OP_CX:
                g.apply_cx(op.a, op.b)
    tol = 1e-12 if prec == 64 else 1e-5
    # double-float: the f64 <-> (hi, lo) conversions truncate, so the norm
    # drifts down by ~6e-15 per gate; 3600 gates at 30 qubits stay below 1e-10
    norm_tol = 1e-10 if fast else tol * 10
    assert abs(g.norm_sqr() - 1) < norm_tol
    assert abs(g.prob_one(n - 1)) < tol
    s = g.sample(1000, 1)
    assert np.all(s == 0)
    g.close()
