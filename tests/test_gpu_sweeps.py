"""Multi-op sweeps and the fast arithmetic modes.

Exact mode: a sweep applies its ops in program order (permutations may move
past disjoint ops, which is exact), so the state must stay bit-identical to
the oracle applying the same ops one by one. Fast mode (FMA for f32,
double-float on the FP32 pipe for f64) must stay within 1e-12 (f64) and
1e-5 (f32) of the exact oracle.
"""

import numpy as np
import pytest

from helpers import bits_equal, rand_matrix, rand_state
from zeno_gb300 import circuit as C

pytestmark = pytest.mark.gpu


def replay(zc, oracle, n, prec, ops, flags, amps=None):
    g = zc.CudaBackend(n, prec, flags)
    o = oracle.State(n, prec)
    if amps is not None:
        g.load_state(amps)
        o.load(amps)
    for op in ops:
        kind = op[0]
        if kind == "u":
            g.apply_unitary(op[1], op[2])
            o.apply_unitary(op[1], op[2])
        elif kind == "d":
            g.apply_diagonal(op[1], op[2])
            o.apply_diagonal(op[1], op[2])
        elif kind == "cx":
            g.apply_cx(op[1], op[2])
            o.apply_cx(op[1], op[2])
        elif kind == "swap":
            swap = np.zeros((4, 4), complex)
            for c in range(4):
                swap[((c & 1) << 1) | ((c >> 1) & 1), c] = 1
            g.apply_swap(op[1], op[2])
            o.apply_unitary(sorted(op[1:3]), swap)
    return g, o


def random_ops(n, count, seed, with_kq=True):
    rng = np.random.default_rng(seed)
    ops = []
    for i in range(count):
        r = rng.integers(0, 10)
        if r < 4:
            q = int(rng.integers(0, n))
            ops.append(("u", [q], rand_matrix(2, seed * 1000 + i)))
        elif r < 5:
            k = int(rng.integers(1, 5))
            qs = sorted(int(x) for x in rng.choice(n, k, replace=False))
            ops.append(("d", qs, rand_state(k, seed * 1000 + i)))
        elif r < 7:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(("cx", a, b))
        elif r < 8:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(("swap", a, b))
        elif with_kq and r < 9:
            qs = sorted(int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(("u", qs, rand_matrix(4, seed * 1000 + i)))
        else:
            q = int(rng.integers(0, n))
            ops.append(("d", [q], rand_state(1, i)))
    return ops


@pytest.mark.parametrize("prec", (64, 32))
@pytest.mark.parametrize("n", (4, 7, 11, 14, 17))
def test_forced_sweeps_bit_exact(zc, oracle, prec, n):
    amps = rand_state(n, n, normalize=True)
    ops = random_ops(n, 160, 10 + n)
    g, o = replay(zc, oracle, n, prec, ops, zc.FLAG_FORCE_SWEEPS, amps)
    a, b = g.statevector(), o.statevector()
    assert bits_equal(a, b), "max |d| = %g" % np.abs(a - b).max()
    c = g.counters()
    assert c["launches"] < len(ops), c  # ops were batched
    g.close()


@pytest.mark.parametrize("prec", (64, 32))
def test_default_sweeps_20q_circuit(zc, oracle, prec):
    p = C.matching_circuit(20, 12, 7).to_program()
    r = zc.run(p, shots=2048, seed=7, precision=prec, statevector=True)
    ref, _, sv, _ = oracle.run(p, prec=prec, shots=2048, seed=7, statevector=True)
    assert bits_equal(r.statevector, sv)
    assert r.counts == ref
    assert r.sweeps < 12 * 30, r.sweeps  # far fewer passes than ops


def test_sweeps_with_reads_between(zc, oracle):
    """Flush points (prob_one, measure, norm) must see every queued op."""
    n = 16
    amps = rand_state(n, 3, normalize=True)
    ops = random_ops(n, 60, 99, with_kq=False)
    g, o = replay(zc, oracle, n, 64, ops[:30], zc.FLAG_EXACT, amps)
    assert g.prob_one(5) == o.prob_one(5)
    assert g.measure(9, 0.4) == o.measure(9, 0.4)
    for op in ops[30:]:
        if op[0] == "u":
            g.apply_unitary(op[1], op[2]); o.apply_unitary(op[1], op[2])
        elif op[0] == "d":
            g.apply_diagonal(op[1], op[2]); o.apply_diagonal(op[1], op[2])
        elif op[0] == "cx":
            g.apply_cx(op[1], op[2]); o.apply_cx(op[1], op[2])
    assert g.norm_sqr() == o.norm_sqr()
    assert bits_equal(g.statevector(), o.statevector())
    g.close()


@pytest.mark.parametrize("n", (6, 15, 20))
def test_fast_mode_f64_within_1e12(zc, oracle, n):
    amps = rand_state(n, 5, normalize=True)
    ops = [op for op in random_ops(n, 200, 40 + n) if not (op[0] == "u" and len(op[1]) > 1)]
    # unitary matrices for realistic magnitudes
    ops = [("u", op[1], np.linalg.qr(op[2])[0]) if op[0] == "u" else op for op in ops]
    ops = [("d", op[1], op[2] / np.abs(op[2])) if op[0] == "d" else op for op in ops]
    for flags in (zc.FLAG_FAST, zc.FLAG_FAST | zc.FLAG_FORCE_SWEEPS, zc.FLAG_FAST | zc.FLAG_NO_SWEEPS):
        g, o = replay(zc, oracle, n, 64, ops, flags, amps)
        d = np.abs(g.statevector() - o.statevector()).max()
        assert d < 1e-12, (flags, d)
        g.close()


@pytest.mark.parametrize("n", (15, 20))
def test_fast_mode_f64_general_matrices(zc, oracle, n):
    """The fast f64 lowering keeps a one-qubit matrix whole when its phases do
    not split as diagonal * real * diagonal, and uses a general real 2x2 when
    the real factor is not a rotation: both inside register passes, within
    1e-12 of the oracle relative to the largest amplitude."""
    rng = np.random.default_rng(n)
    amps = rand_state(n, 9, normalize=True)
    ops = []
    for i in range(160):
        q = int(rng.integers(0, n))
        u = np.linalg.qr(rand_matrix(2, 7000 + i))[0]
        kind = i % 4
        if kind == 1:
            u = u.copy()
            u[0, 1] *= 1j  # phases no diagonal * real * diagonal gives
        elif kind == 2:
            u = u.copy()
            u[0, 1] *= 0.5  # a real factor that is not a rotation
        ops.append(("u", [q], u))
        if kind == 3:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(("cx", a, b))
    g, o = replay(zc, oracle, n, 64, ops, zc.FLAG_FAST, amps)
    want = o.statevector()
    d = np.abs(g.statevector() - want).max() / np.abs(want).max()
    assert d < 1e-12, d
    g.close()


def test_fast_mode_f32_within_1e5(zc, oracle):
    n = 18
    p = C.matching_circuit(n, 10, 3).to_program()
    exact = oracle.run(p, prec=64, shots=0, statevector=True)[2]
    r = zc.run(p, shots=0, precision=32, statevector=True, flags=zc.FLAG_FAST)
    assert np.abs(r.statevector - exact).max() < 1e-5


@pytest.mark.parametrize("n", (20, 24))
def test_fast_mode_circuit_vs_fp64_oracle(zc, oracle, n):
    """max|d amp| <= 1e-12 and TVD <= 1e-6 against the FP64 oracle."""
    p = C.matching_circuit(n, 12, 11).to_program()
    _, _, sv, _ = oracle.run(p, prec=64, shots=0, statevector=True)
    r = zc.run(p, shots=0, precision=64, statevector=True, flags=zc.FLAG_FAST)
    d = np.abs(r.statevector - sv).max()
    tvd = 0.5 * np.abs(np.abs(r.statevector) ** 2 - np.abs(sv) ** 2).sum()
    assert d < 1e-12 and tvd < 1e-6, (d, tvd)


def test_fast_mode_qft_with_swaps(zc, oracle):
    c, x = C.qft_circuit(16, 5)
    p = c.to_program()
    r = zc.run(p, shots=4096, seed=2, precision=64, statevector=True, flags=zc.FLAG_FAST)
    dim = 1 << 16
    want = np.exp(2j * np.pi * x * np.arange(dim) / dim) / np.sqrt(dim)
    assert np.abs(r.statevector - want).max() < 1e-12


def test_autotuned_runs_stay_bit_exact(zc, oracle):
    """Exact mode: every (fusion, tile shape) the tuner may pick gives the
    oracle's bits at that fusion; the tuner returns the fastest it timed."""
    from zeno_gb300 import autotune as at

    n = 16
    p = C.matching_circuit(n, 6, 9).to_program()
    for k, h in ((1, 4), (2, 7), (3, 5)):
        prog = zc.compile(p, k)
        r = zc.run(p, shots=0, precision=64, statevector=True, flags=zc.FLAG_EXACT | zc.FLAG_FORCE_SWEEPS,
                   program=prog, sweep_high=h)
        _, _, sv, _ = oracle.run(p, prec=64, shots=0, fusion=k, statevector=True)
        assert np.array_equal(r.statevector.view(np.float64), sv.view(np.float64)), (k, h)
    t = at.tune(p, 64, zc.FLAG_FAST, fusions=(1, 2), highs=(0, 5))
    assert min(r["seconds"] for r in t["table"]) == [r["seconds"] for r in t["table"]
                                                      if (r["fusion"], r["max_high"]) == (t["fusion"], t["max_high"])][0]


@pytest.mark.parametrize("n", (9, 16))
def test_fast_mode_f64_dense_blocks_within_1e12(zc, oracle, n):
    """Fast f64 dense k-qubit blocks (k = 2..7, supports spanning low and
    high qubits) run in double-float on the FP32 pipe: within 1e-12 of the
    FP64 oracle, on random unitaries and a random normalised state."""
    rng = np.random.default_rng(100 + n)
    amps = rand_state(n, 13, normalize=True)
    ops = []
    for i in range(24):
        k = 2 + i % 6
        qs = sorted(int(x) for x in rng.choice(n, k, replace=False))
        ops.append(("u", qs, np.linalg.qr(rand_matrix(1 << k, 900 + i))[0]))
        if i % 3 == 0:
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ops.append(("cx", a, b))
    g, o = replay(zc, oracle, n, 64, ops, zc.FLAG_FAST, amps)
    d = np.abs(g.statevector() - o.statevector()).max()
    assert d < 1e-12, d
    g.close()


@pytest.mark.parametrize("fusion", (2, 3, 5))
def test_fast_mode_fused_circuit_vs_fp64_oracle(zc, oracle, fusion):
    """The fused matching circuit at fusion width K in fast f64 (dense blocks
    in double-float) against the oracle's FP64 run at the same K."""
    p = C.matching_circuit(18, 10, 3).to_program()
    _, _, sv, _ = oracle.run(p, prec=64, shots=0, fusion=fusion, statevector=True)
    r = zc.run(p, shots=0, precision=64, fusion=fusion, statevector=True, flags=zc.FLAG_FAST)
    d = np.abs(r.statevector - sv).max()
    tvd = 0.5 * np.abs(np.abs(r.statevector) ** 2 - np.abs(sv) ** 2).sum()
    assert d < 1e-12 and tvd < 1e-6, (fusion, d, tvd)


@pytest.mark.parametrize("prec,tol", ((64, 1e-12), (32, 1e-5)))
def test_fast_mode_deep_circuit_vs_fp64_oracle(zc, oracle, prec, tol):
    """The headline circuit family at its full depth (40 layers of u3 on every
    qubit + matching CX), 22 qubits, fast arithmetic against the FP64 oracle:
    max |d amp| within the fast-mode tolerance, TVD <= 1e-6 for f64."""
    p = C.matching_circuit(22, 40, 7).to_program()
    _, _, sv, _ = oracle.run(p, prec=64, shots=0, statevector=True)
    r = zc.run(p, shots=0, precision=prec, statevector=True, flags=zc.FLAG_FAST)
    d = np.abs(r.statevector - sv).max()
    tvd = 0.5 * np.abs(np.abs(r.statevector) ** 2 - np.abs(sv) ** 2).sum()
    assert d < tol, (prec, d)
    if prec == 64:
        assert tvd < 1e-6, tvd


def test_qft_22q_exact_and_fast(zc, oracle):
    """QFT with the final SWAP network at 22 qubits: exact mode bit-identical
    to the oracle (state and counts); fast f64 within 1e-12 of the oracle's
    FP64 state. Both sit within a few 1e-12 of the DFT of the prepared basis
    state (253 controlled phases with rounded cos/sin accumulate that)."""
    c, x = C.qft_circuit(22, 9)
    p = c.to_program()
    ref, _, sv, _ = oracle.run(p, prec=64, shots=8192, seed=4, statevector=True)
    ex = zc.run(p, shots=8192, seed=4, precision=64, statevector=True, flags=zc.FLAG_EXACT)
    assert bits_equal(ex.statevector, sv)
    assert ex.counts == ref
    fa = zc.run(p, shots=0, precision=64, statevector=True, flags=zc.FLAG_FAST)
    assert np.abs(fa.statevector - sv).max() < 1e-12
    dim = 1 << 22
    want = np.exp(2j * np.pi * x * np.arange(dim) / dim) / np.sqrt(dim)
    assert np.abs(sv - want).max() < 1e-11 and np.abs(fa.statevector - want).max() < 1e-11


def _apply(g, o, op):
    if op[0] == "u":
        g.apply_unitary(op[1], op[2])
        o.apply_unitary(op[1], op[2])
    elif op[0] == "d":
        g.apply_diagonal(op[1], op[2])
        o.apply_diagonal(op[1], op[2])
    elif op[0] == "cx":
        g.apply_cx(op[1], op[2])
        o.apply_cx(op[1], op[2])
    else:
        swap = np.zeros((4, 4), complex)
        for c in range(4):
            swap[((c & 1) << 1) | ((c >> 1) & 1), c] = 1
        g.apply_swap(op[1], op[2])
        o.apply_unitary(sorted(op[1:3]), swap)


@pytest.mark.parametrize("n", (16, 19))
def test_fast_f64_sweeps_blocks_and_reads_interleaved(zc, oracle, n):
    """Fast f64 across the boundaries of its sweeps: runs of sweeps hand the
    state over as packed double-float pairs, and a dense 2- or 3-qubit block
    or a read (prob_one, measure, norm) in the middle of the program first
    turns it back into f64. Every read and the final state stay within 1e-12
    of the FP64 oracle."""
    rng = np.random.default_rng(n)
    amps = rand_state(n, 70 + n, normalize=True)
    ops = random_ops(n, 240, 90 + n)
    ops = [("u", op[1], np.linalg.qr(op[2])[0]) if op[0] == "u" else op for op in ops]
    ops = [("d", op[1], op[2] / np.abs(op[2])) if op[0] == "d" else op for op in ops]
    g = zc.CudaBackend(n, 64, zc.FLAG_FAST)
    o = oracle.State(n, 64)
    g.load_state(amps)
    o.load(amps)
    reads = 0
    for i, op in enumerate(ops):
        _apply(g, o, op)
        if i % 60 == 30:  # a three-qubit dense block between sweeps
            qs = sorted(int(x) for x in rng.choice(n, 3, replace=False))
            _apply(g, o, ("u", qs, np.linalg.qr(rand_matrix(8, 5000 + i))[0]))
        if i % 40 == 39:
            q = int(rng.integers(0, n))
            p = o.prob_one(q)
            assert abs(g.prob_one(q) - p) <= 1e-12, (i, q)
            if i % 80 == 79:
                u = 0.5 if abs(p - 0.5) > 1e-6 else 0.25
                assert g.measure(q, u) == o.measure(q, u), (i, q)
            assert abs(g.norm_sqr() - o.norm_sqr()) <= 1e-12, i
            reads += 1
    assert reads == 6
    d = np.abs(g.statevector() - o.statevector()).max()
    assert d < 1e-12, d
    c = g.counters()
    assert c["sweeps"] > 0
    g.close()
