"""Pin the CPU oracle against the reference's own known answers.

Ports of zeno's tests (tests/reference.rs, tests/analytic.rs, tests/noise.rs,
src/state.rs, src/sample.rs, src/mem.rs) run against the C restatement, plus
the expected outputs the reference's example programs state. These run on
CPU only.
"""

import math

import numpy as np
import pytest

import refmats
from helpers import Sm64, bits_equal, max_delta, program_from_json, rand_state, supports
from zeno_gb300 import circuit as C
from zeno_gb300.rng import Xoshiro256pp, splitmix64


def test_rng_streams_agree(oracle):
    """The oracle's xoshiro256++/splitmix64 and the Python generator stream agree."""
    import ctypes

    for seed in (0, 1, 7, 0xDEADBEEF, 2**64 - 1):
        assert oracle.lib().zo_splitmix64(seed) == splitmix64(seed)
    # Drive the oracle's sampler: identical draws imply identical streams.
    st = oracle.State(3)
    h = refmats.ref_gate("h")
    for q in range(3):
        st.apply_unitary([q], h)
    a = st.sample(64, 42)
    r = Xoshiro256pp(42)
    us = sorted(r.f64() * 1.0 for _ in range(64))
    want = [min(int(u * 8), 7) for u in us]
    assert list(a) == want


def test_gen_range_is_unbiased_in_range():
    r = Xoshiro256pp(3)
    xs = [r.range(1, 16) for _ in range(20000)]
    assert min(xs) == 1 and max(xs) == 15
    counts = np.bincount(xs, minlength=16)[1:]
    assert counts.min() > 1100 and counts.max() < 1600


def test_gate_library_matches_hand_coded_matrices(oracle):
    """tests/reference.rs:472-506."""
    rng = Sm64(0x51DECAFE)
    for name, arity, npar in refmats.NATIVE:
        for _ in range(3):
            params = [rng.angle() for _ in range(npar)]
            kind, m = oracle.gate_matrix(name, params)
            lib = m if kind == 0 else np.diag(m)
            assert max_delta(lib.reshape(-1), refmats.ref_gate(name, params).reshape(-1)) < 1e-14, name


def test_gate_unitarity(oracle):
    """src/gates.rs:209-272."""
    for name, arity, npar in refmats.NATIVE:
        kind, m = oracle.gate_matrix(name, [0.3, 1.1, -0.7][:npar])
        u = m if kind == 0 else np.diag(m)
        assert np.abs(u @ u.conj().T - np.eye(len(u))).max() < 1e-12


@pytest.mark.parametrize("name,arity,npar", refmats.NATIVE)
def test_every_gate_every_argument_order(oracle, name, arity, npar):
    """tests/reference.rs:508-556: fusion 0 and 5, 1e-12."""
    orders = {1: [[0], [2], [3]], 2: [[0, 1], [1, 0], [3, 1], [2, 3], [3, 0]],
              3: [[0, 1, 2], [3, 0, 2], [2, 3, 0], [1, 3, 2]]}[arity]
    rng = Sm64(0xA5A50001 + arity * 131 + npar)
    for qs in orders:
        params = [rng.angle() for _ in range(npar)]
        c = C.Circuit(4)
        for q in range(4):
            c.u(q, rng.angle(), rng.angle(), rng.angle())
        c.gate(name, qs, params)
        want = refmats.simulate(c.to_program())
        for fusion in (0, 5):
            _, _, sv, _ = oracle.run(c.to_program(), shots=0, fusion=fusion, statevector=True)
            assert max_delta(sv, want) < 1e-12, (name, qs, fusion)


def _mixed(n, count, seed, barriers=True):
    pool = [g for g in refmats.NATIVE if g[0] not in ("id", "u0") and g[1] <= n]
    rng = Sm64(seed)
    c = C.Circuit(n)
    for _ in range(count):
        name, arity, npar = pool[rng.below(len(pool))]
        qs = []
        while len(qs) < arity:
            q = rng.below(n)
            if q not in qs:
                qs.append(q)
        c.gate(name, qs, [rng.angle() for _ in range(npar)])
        if barriers and rng.below(8) == 0:
            c.barrier()
    return c


@pytest.mark.parametrize("n", range(2, 11))
def test_random_circuits_all_fusion_levels(oracle, n):
    """tests/reference.rs:601-617: fusion 0..6 within 1e-10, norm within 1e-12."""
    for c in (C.random_circuit(n, 20, 1000 + n), _mixed(n, 60, 9000 + n)):
        want = refmats.simulate(c.to_program())
        for fusion in range(7):
            _, _, sv, _ = oracle.run(c.to_program(), shots=0, fusion=fusion, statevector=True)
            assert abs(np.linalg.norm(sv) - 1) < 1e-12
            assert max_delta(sv, want) < 1e-10, (n, fusion)


def test_f32_tracks_f64(oracle):
    """tests/reference.rs:621-648: f32 within 2e-4."""
    for n in (4, 8, 10):
        for c in (C.random_circuit(n, 20, 1000 + n), _mixed(n, 60, 9000 + n)):
            want = refmats.simulate(c.to_program())
            for fusion in (0, 5):
                _, _, sv, _ = oracle.run(c.to_program(), prec=32, shots=0, fusion=fusion, statevector=True)
                assert max_delta(sv, want) < 2e-4


def test_diagonal_ladder_and_flushes(oracle):
    """tests/reference.rs:652-716."""
    n = 6
    c = C.Circuit(n)
    for q in range(n):
        c.h(q)
    rng = Sm64(0xD1A60001)
    pool = [("z", 1, 0), ("s", 1, 0), ("sdg", 1, 0), ("t", 1, 0), ("tdg", 1, 0), ("rz", 1, 1), ("p", 1, 1),
            ("cz", 2, 0), ("cp", 2, 1), ("crz", 2, 1), ("rzz", 2, 1)]
    for _ in range(40):
        name, arity, npar = pool[rng.below(len(pool))]
        qs = []
        while len(qs) < arity:
            q = rng.below(n)
            if q not in qs:
                qs.append(q)
        c.gate(name, qs, [rng.angle() for _ in range(npar)])
    c.cp(5, 2, 0.4).crz(4, 1, 0.8).rzz(3, 0, 1.1).gate("cu1", [4, 0], [0.6]).crz(1, 5, -0.9)
    want = refmats.simulate(c.to_program())
    for fusion in range(7):
        _, _, sv, _ = oracle.run(c.to_program(), shots=0, fusion=fusion, statevector=True)
        assert max_delta(sv, want) < 1e-10
    c = C.Circuit(8)
    for r in range(4):
        th = 0.3 + r * 0.17
        c.ccx(0, 1, 2).u(3, th, 0.2, 0.9).cx(2, 3).h(0).swap(1, 3)
        c.ccx(4, 5, 6).u(7, th + 0.05, 1.1, 0.4).cx(6, 7).h(4).swap(5, 7)
    want = refmats.simulate(c.to_program())
    comp = oracle.compile(c.to_program(), 5)
    assert comp.stats["max_fused"] <= 5 and comp.stats["output_ops"] >= 2
    for fusion in range(7):
        _, _, sv, _ = oracle.run(c.to_program(), shots=0, fusion=fusion, statevector=True)
        assert max_delta(sv, want) < 1e-10


def test_harness_detects_injected_errors(oracle):
    """tests/reference.rs:558-599: a sign-flipped S or swapped CX must be visible."""
    c = C.Circuit(1)
    c.h(0).s(0)
    _, _, sv, _ = oracle.run(c.to_program(), shots=0, statevector=True)
    good = refmats.apply_dense(refmats.apply_dense(np.array([1, 0], complex), 1, [0], refmats.ref_gate("h")), 1,
                               [0], refmats.ref_gate("s"))
    bad = refmats.apply_dense(refmats.apply_dense(np.array([1, 0], complex), 1, [0], refmats.ref_gate("h")), 1,
                              [0], refmats.ref_gate("sdg"))
    assert max_delta(sv, good) < 1e-12 and max_delta(sv, bad) > 0.5
    c = C.Circuit(2)
    c.u(0, 0.9, 0.4, 1.3).u(1, 0.5, 2.1, -0.7).cx(0, 1)
    _, _, sv, _ = oracle.run(c.to_program(), shots=0, statevector=True)
    d = C.Circuit(2)
    d.u(0, 0.9, 0.4, 1.3).u(1, 0.5, 2.1, -0.7).cx(1, 0)
    assert max_delta(sv, refmats.simulate(d.to_program())) > 0.1


def test_qft5_dft_formula(oracle):
    """tests/analytic.rs:189-238."""
    n, dim = 5, 32
    for x in (0, 1, 5, 19, 31):
        c = C.Circuit(n)
        for q in range(n):
            if (x >> q) & 1:
                c.x(q)
        for i in range(n - 1, -1, -1):
            c.h(i)
            for j in range(i - 1, -1, -1):
                c.cp(j, i, math.pi / (1 << (i - j)))
        _, _, sv, _ = oracle.run(c.to_program(), shots=0, statevector=True)
        assert max_delta(sv, refmats.simulate(c.to_program())) < 1e-12
        for j in range(dim):
            rev = int(format(j, "05b")[::-1], 2)
            want = complex(math.cos(2 * math.pi * x * j / dim), math.sin(2 * math.pi * x * j / dim)) / math.sqrt(dim)
            assert abs(sv[rev] - want) < 1e-12


def six_sigma(count, shots, p):
    mean = shots * p
    sigma = math.sqrt(shots * p * (1 - p))
    assert abs(count - mean) <= 6 * sigma + 1e-9, (count, mean, sigma)


def test_ghz12_two_branches(oracle):
    """tests/analytic.rs:167-187."""
    c = C.Circuit(12)
    c.h(0)
    for q in range(11):
        c.cx(q, q + 1)
    c.measure_all()
    counts, _, _, _ = oracle.run(c.to_program(), shots=20000, seed=41)
    assert set(counts) == {"0" * 12, "1" * 12}
    six_sigma(counts["0" * 12], 20000, 0.5)


def test_examples_known_answers(oracle, examples):
    """The expected outputs stated by the reference's examples/*.qasm."""
    for name, d in examples.items():
        p = program_from_json(d)
        counts, _, _, _ = oracle.run(p, shots=4000, seed=11, fusion=1)
        exp = d["expected"]
        assert sum(counts.values()) == 4000
        if exp["kind"] == "exact":
            assert counts == {exp["keys"][0]: 4000}, (name, counts)
        elif exp["kind"] == "support":
            assert set(counts) <= set(exp["keys"]), (name, counts)
        else:
            six_sigma(counts[exp["keys"][0]], 4000, exp["p"])


def test_analytic_statistics(oracle):
    """tests/analytic.rs 6-sigma checks: uniform superposition, reset after
    entanglement, mid-circuit measurement feeding a later gate."""
    shots = 16000
    c = C.Circuit(4)
    for q in range(4):
        c.h(q)
    c.measure_all()
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=31)
    assert len(counts) == 16
    for key in counts:
        six_sigma(counts[key], shots, 1 / 16)
    # reset of one half of a Bell pair: that qubit reads 0, the other stays uniform
    c = C.Circuit(2)
    c.h(0).cx(0, 1).reset(0).measure(0, 0).measure(1, 1)
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=32)
    assert set(counts) <= {"00", "10"}, counts
    six_sigma(counts.get("10", 0), shots, 0.5)
    # a mid-circuit outcome copied forward by CX: both bits always agree
    c = C.Circuit(2)
    c.h(0).measure(0, 0).cx(0, 1).measure(1, 1)
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=33)
    assert set(counts) <= {"00", "11"}, counts
    six_sigma(counts.get("11", 0), shots, 0.5)


def test_same_seed_determinism(oracle):
    c = C.random_circuit(6, 8, 3)
    c.measure_all()
    a = oracle.run(c.to_program(), shots=1000, seed=99)[0]
    b = oracle.run(c.to_program(), shots=1000, seed=99)[0]
    assert a == b


def test_sampler_bell_balance(oracle):
    """src/sample.rs:128-144."""
    st = oracle.State(2)
    st.apply_unitary([0], refmats.ref_gate("h"))
    kind, cx = oracle.gate_matrix("cx")
    st.apply_unitary([0, 1], cx)
    s = st.sample(100000, 7)
    ones = int((s == 3).sum())
    assert ones + int((s == 0).sum()) == 100000
    assert abs(ones / 1e5 - 0.5) < 0.01


def test_mem_capacity_math(oracle):
    """src/mem.rs:133-151."""
    b = 24 << 30
    assert oracle.max_qubits(b, 64) == 30 and oracle.max_qubits(b, 32) == 31
    assert oracle.state_bytes(30, 64) == 16 << 30 and oracle.state_bytes(30, 32) == 8 << 30


def test_prob_one_collapse_norm(oracle):
    st = oracle.State(2)
    st.apply_unitary([0], refmats.ref_gate("h"))
    _, cx = oracle.gate_matrix("cx")
    st.apply_unitary([0, 1], cx)
    p1 = st.prob_one(0)
    assert abs(p1 - 0.5) < 1e-12
    assert st.measure(0, 0.25)
    assert abs(st.norm_sqr() - 1) < 1e-12
    assert abs(abs(st.statevector()[3]) - 1) < 1e-12


class _N:
    def __init__(self, **kw):
        for f in ("depolarizing_1q", "depolarizing_2q", "bit_flip", "phase_flip", "amplitude_damping",
                  "readout_flip_0to1", "readout_flip_1to0"):
            setattr(self, f, kw.get(f, 0.0))


def test_noise_closed_forms(oracle):
    """tests/noise.rs: bit flip P=p, depolarizing 2p/3, damping (1-g)^k, readout."""
    shots = 20000
    c = C.Circuit(1)
    c.x(0).measure(0, 0)
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=5, noise=_N(bit_flip=0.1))
    six_sigma(counts.get("0", 0), shots, 0.1)
    c = C.Circuit(1)
    c.gate("sx", [0]).gate("sxdg", [0]).measure(0, 0)
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=6, noise=_N(depolarizing_1q=0.3))
    # two noisy gates: P(1) = 1 - (1 - 2p/3)^2 - ... exact for two independent channels:
    q = 2 * 0.3 / 3
    six_sigma(counts.get("1", 0), shots, 2 * q * (1 - q))
    c = C.Circuit(1)
    c.x(0)
    for _ in range(3):
        c.gate("sx", [0]).gate("sxdg", [0])
    c.measure(0, 0)
    g = 0.05
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=8, noise=_N(amplitude_damping=g))
    six_sigma(counts.get("1", 0), shots, _damp_p1(g))
    c2 = C.Circuit(1)
    c2.x(0).measure(0, 0)
    counts, _, _, _ = oracle.run(c2.to_program(), shots=shots, seed=9, noise=_N(readout_flip_1to0=0.2))
    six_sigma(counts.get("0", 0), shots, 0.2)


def test_noise_two_qubit_and_phase_closed_forms(oracle):
    """tests/noise.rs:312-384: a depolarizing hit on CX draws one of the 15
    non-identity Pauli strings, so |00> changes with probability 12p/15 and
    the Bell parity flips with 8p/15 (<ZZ> = 1 - 16p/15); a phase flip after
    H shows up as P(1) = p once RY(-pi/2) maps |+>, |-> to |0>, |1> (H H
    would cancel in the compiler and carry no noise)."""
    shots, p = 20000, 0.3
    c = C.Circuit(2)
    c.cx(0, 1).measure(0, 0).measure(1, 1)
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=21, noise=_N(depolarizing_2q=p))
    six_sigma(shots - counts.get("00", 0), shots, 12 * p / 15)
    c = C.Circuit(2)
    c.h(0).cx(0, 1).measure(0, 0).measure(1, 1)
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=22, noise=_N(depolarizing_2q=p))
    odd = counts.get("01", 0) + counts.get("10", 0)
    six_sigma(odd, shots, 8 * p / 15)
    c = C.Circuit(1)
    c.h(0).ry(0, -math.pi / 2).measure(0, 0)
    counts, _, _, _ = oracle.run(c.to_program(), shots=shots, seed=23, noise=_N(phase_flip=0.2))
    six_sigma(counts.get("1", 0), shots, 0.2)


def _damp_p1(g):
    """P(1) after x, then 3 x (sx, sxdg) pairs with damping after each of the 7 gates.

    Computed by exact density-matrix evolution (independent of the trajectory code)."""
    X = np.array([[0, 1], [1, 0]], complex)
    SX = refmats.ref_gate("sx")
    SXD = refmats.ref_gate("sxdg")
    K0 = np.array([[1, 0], [0, math.sqrt(1 - g)]], complex)
    K1 = np.array([[0, math.sqrt(g)], [0, 0]], complex)
    rho = np.array([[1, 0], [0, 0]], complex)

    def gate(U):
        nonlocal rho
        rho = U @ rho @ U.conj().T
        rho = K0 @ rho @ K0.conj().T + K1 @ rho @ K1.conj().T

    gate(X)
    for _ in range(3):
        gate(SX)
        gate(SXD)
    return float(rho[1, 1].real)


def test_noisy_runs_are_seed_deterministic(oracle):
    c = C.matching_circuit(6, 4, 17)
    n = _N(depolarizing_1q=0.01, depolarizing_2q=0.05, amplitude_damping=0.02, readout_flip_0to1=0.02,
           readout_flip_1to0=0.02)
    a = oracle.run(c.to_program(), shots=300, seed=3, noise=n)[0]
    oracle.set_threads(1)
    b = oracle.run(c.to_program(), shots=300, seed=3, noise=n)[0]
    oracle.set_threads(0)
    assert a == b
