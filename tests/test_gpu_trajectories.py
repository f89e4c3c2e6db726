"""Batched noisy trajectories (one launch for all shots).

The engine draws from per-trajectory Philox streams, so counts agree with
zeno's per-shot replay in distribution, not bit for bit — the same standard
the reference applies to its CPU-vs-Metal noisy parity (TVD < 0.05,
tests/noise.rs:703-735). Closed-form channel values are checked at 6 sigma
like tests/noise.rs:45-384.
"""

import math

import numpy as np
import pytest

import refmats
from zeno_gb300 import circuit as C

pytestmark = pytest.mark.gpu


def six_sigma(count, shots, p):
    sigma = math.sqrt(shots * p * (1 - p))
    assert abs(count - shots * p) <= 6 * sigma + 1e-9, (count, shots * p, sigma)


def tvd(a, b):
    na, nb = sum(a.values()), sum(b.values())
    keys = set(a) | set(b)
    return 0.5 * sum(abs(a.get(k, 0) / na - b.get(k, 0) / nb) for k in keys)


def batched(zc, p, shots, seed, noise):
    r = zc.run(p, shots=shots, seed=seed, precision=32, noise=noise)
    assert r.batched, "expected the batched trajectory engine"
    assert sum(r.counts.values()) == shots
    return r


def test_bit_flip_and_readout(zc):
    shots = 40000
    c = C.Circuit(1)
    c.x(0).measure(0, 0)
    r = batched(zc, c.to_program(), shots, 1, zc.NoiseModel(bit_flip=0.1))
    six_sigma(r.counts.get("0", 0), shots, 0.1)
    r = batched(zc, c.to_program(), shots, 2, zc.NoiseModel(readout_flip_1to0=0.2))
    six_sigma(r.counts.get("0", 0), shots, 0.2)


def test_depolarizing_two_thirds(zc):
    """P(flip) of a depolarized basis state = 2p/3 per gate (tests/noise.rs:88-112)."""
    shots = 40000
    c = C.Circuit(1)
    c.gate("sx", [0]).gate("sxdg", [0]).measure(0, 0)
    r = batched(zc, c.to_program(), shots, 3, zc.NoiseModel(depolarizing_1q=0.3))
    q = 2 * 0.3 / 3
    six_sigma(r.counts.get("1", 0), shots, 2 * q * (1 - q))


def test_two_qubit_depolarizing(zc):
    """12p/15 of the 15 Pauli strings flip a given qubit of |00> ... on CX."""
    shots = 40000
    c = C.Circuit(2)
    c.cx(0, 1).measure_all()
    p = 0.3
    r = batched(zc, c.to_program(), shots, 4, zc.NoiseModel(depolarizing_2q=p))
    # qubit 1 ends in |1> when its Pauli is X or Y: 8 of 15 strings
    ones_q1 = sum(v for k, v in r.counts.items() if k[0] == "1")
    six_sigma(ones_q1, shots, p * 8 / 15)


def _damp_chain(g, gates):
    K0 = np.array([[1, 0], [0, math.sqrt(1 - g)]], complex)
    K1 = np.array([[0, math.sqrt(g)], [0, 0]], complex)
    rho = np.array([[1, 0], [0, 0]], complex)
    for U in gates:
        rho = U @ rho @ U.conj().T
        rho = K0 @ rho @ K0.conj().T + K1 @ rho @ K1.conj().T
    return float(rho[1, 1].real)


def test_amplitude_damping_density_matrix(zc):
    shots = 40000
    g = 0.05
    c = C.Circuit(1)
    c.x(0)
    gates = [refmats.ref_gate("x")]
    for _ in range(3):
        c.gate("sx", [0]).gate("sxdg", [0])
        gates += [refmats.ref_gate("sx"), refmats.ref_gate("sxdg")]
    c.measure(0, 0)
    r = batched(zc, c.to_program(), shots, 5, zc.NoiseModel(amplitude_damping=g))
    six_sigma(r.counts.get("1", 0), shots, _damp_chain(g, gates))


def test_damping_on_superposition(zc):
    """Damping after H: P(1) = (1 - g) / 2 (tests/noise.rs:114-182)."""
    shots = 40000
    g = 0.3
    c = C.Circuit(1)
    c.h(0).measure(0, 0)
    r = batched(zc, c.to_program(), shots, 6, zc.NoiseModel(amplitude_damping=g))
    six_sigma(r.counts.get("1", 0), shots, (1 - g) / 2)


def test_distribution_matches_per_shot_oracle(zc, oracle):
    noise = zc.NoiseModel(depolarizing_1q=0.02, depolarizing_2q=0.05, amplitude_damping=0.03,
                          bit_flip=0.01, phase_flip=0.02, readout_flip_0to1=0.02, readout_flip_1to0=0.02)
    c = C.matching_circuit(6, 5, 31)
    shots = 30000
    mine = batched(zc, c.to_program(), shots, 9, noise).counts
    ref = oracle.run(c.to_program(), prec=64, shots=shots, seed=9, noise=noise)[0]
    assert tvd(mine, ref) < 0.05, tvd(mine, ref)


def test_config_shape_runs_and_is_deterministic(zc):
    """16 qubits, depth 20, the 1e-3 / 1e-2 / 1e-3 / 2% model, 4096 trajectories."""
    noise = zc.NoiseModel(depolarizing_1q=1e-3, depolarizing_2q=1e-2, amplitude_damping=1e-3,
                          readout_flip_0to1=0.02, readout_flip_1to0=0.02)
    p = C.matching_circuit(16, 20, 7).to_program()
    a = batched(zc, p, 4096, 11, noise)
    b = batched(zc, p, 4096, 11, noise)
    assert a.counts == b.counts
    assert a.launches <= 2
    c = batched(zc, p, 4096, 12, noise)
    assert c.counts != a.counts


def test_noiseless_limit_matches_ideal_distribution(zc, oracle):
    """Readout noise only: the output is the ideal distribution with flips."""
    c = C.matching_circuit(4, 3, 2)
    shots = 40000
    noise = zc.NoiseModel(readout_flip_0to1=1e-12)
    mine = batched(zc, c.to_program(), shots, 3, noise).counts
    ideal = oracle.run(c.to_program(), prec=64, shots=shots, seed=3)[0]
    assert tvd(mine, ideal) < 0.04


def test_per_shot_flag_reproduces_oracle_stream(zc, oracle):
    noise = zc.NoiseModel(depolarizing_1q=0.02, amplitude_damping=0.05, readout_flip_0to1=0.05)
    c = C.matching_circuit(4, 3, 17)
    r = zc.run(c.to_program(), shots=300, seed=5, precision=32, noise=noise, flags=zc.FLAG_PER_SHOT)
    assert not r.batched
    ref = oracle.run(c.to_program(), prec=32, shots=300, seed=5, noise=noise)[0]
    assert r.counts == ref


def _bits(counts, n):
    """Shots as an (N, n) 0/1 array; bit j = clbit j (keys print clbit n-1 first)."""
    rows = []
    for k, v in counts.items():
        b = [(int(k, 2) >> j) & 1 for j in range(n)]
        rows.extend([b] * v)
    return np.array(rows, dtype=np.int8)


def test_config_shape_matches_per_shot_oracle(zc, oracle):
    """The trajectory workload at its own shape — 16 qubits, depth 20 (u3 +
    matching CX), depolarizing 1e-3 / 1e-2, amplitude damping 1e-3 per
    touched qubit after each gate, 2% readout — against the oracle's
    per-shot replay (zeno's run_per_shot). 2^16 outcomes are far more than
    any affordable shot count resolves, so the comparison is on what the
    shots do resolve: every qubit's P(1) at 6 sigma, and the 16-outcome
    distribution of each block of four qubits by TVD within 6 sigma of the
    TVD that sampling alone gives (the reference's own noisy-parity check
    compares 16-outcome distributions by TVD, tests/noise.rs:703-735)."""
    noise = zc.NoiseModel(depolarizing_1q=1e-3, depolarizing_2q=1e-2, amplitude_damping=1e-3,
                          readout_flip_0to1=0.02, readout_flip_1to0=0.02)
    n = 16
    p = C.matching_circuit(n, 20, 7).to_program()
    ng, no = 1 << 17, 2048
    g = _bits(batched(zc, p, ng, 21, noise).counts, n)
    o = _bits(oracle.run(p, prec=32, shots=no, seed=22, noise=noise)[0], n)
    assert g.shape == (ng, n) and o.shape == (no, n)
    _agree(g, o, n)


def _agree(g, o, n):
    """Shots of the batched engine (g) and of the per-shot oracle (o) agree:
    every qubit's P(1) at 6 sigma, and each block of four qubits' 16-outcome
    distribution by TVD within 6 sigma of the TVD sampling alone gives."""
    ng, no = len(g), len(o)
    pg, po = g.mean(axis=0), o.mean(axis=0)
    for q in range(n):
        sig = math.sqrt(max(pg[q] * (1 - pg[q]), 1e-12) * (1.0 / ng + 1.0 / no))
        assert abs(pg[q] - po[q]) <= 6 * sig, (q, pg[q], po[q], sig)
    w = 1 << np.arange(4)
    for b0 in range(0, n - 3, 4):
        hg = np.bincount(g[:, b0:b0 + 4] @ w, minlength=16) / ng
        ho = np.bincount(o[:, b0:b0 + 4] @ w, minlength=16) / no
        d = 0.5 * np.abs(hg - ho).sum()
        var = hg * (1 - hg) * (1.0 / ng + 1.0 / no)  # variance of each outcome's difference
        mean = 0.5 * np.sum(np.sqrt(2 / np.pi * var))  # E|N(0, var)| = sqrt(2 var / pi)
        std = 0.5 * np.sqrt(np.sum((1 - 2 / np.pi) * var))
        assert d <= mean + 6 * std, (b0, d, mean, std)


@pytest.mark.parametrize("n", (13, 14, 15))
def test_noisy_13_to_15_qubits_match_per_shot_oracle(zc, oracle, n):
    """Noisy circuits of 13-15 qubits, with noise strong enough that
    depolarizing, both flips and damping all fire, against the oracle's
    per-shot replay: per-qubit marginals and four-qubit blocks."""
    noise = zc.NoiseModel(depolarizing_1q=0.01, depolarizing_2q=0.03, amplitude_damping=0.02, bit_flip=0.005,
                          phase_flip=0.01, readout_flip_0to1=0.02, readout_flip_1to0=0.02)
    p = C.matching_circuit(n, 4, 40 + n).to_program()
    ng, no = 1 << 16, 2048
    g = _bits(batched(zc, p, ng, 31, noise).counts, n)
    o = _bits(oracle.run(p, prec=32, shots=no, seed=32, noise=noise)[0], n)
    assert g.shape == (ng, n) and o.shape == (no, n)
    _agree(g, o, n)
