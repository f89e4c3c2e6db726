"""Parity at the headline size through a size-independent property.

The oracle cannot hold a 30-qubit state in the time a test has, so the
headline circuit (30 qubits, depth 40, u3 + matching CX, f64, fast
arithmetic) is checked by a round trip: the circuit followed by its inverse
must return |0...0>. The inverse reverses the gate order, maps
u3(theta, phi, lambda) to u3(-theta, -lambda, -phi) (its adjoint) and keeps
CX (self-inverse); the construction itself is checked on the CPU against the
oracle. Collected last: the 16 GiB state is the largest any test allocates.
"""

import numpy as np
import pytest

from zeno_gb300 import circuit as C


def inverse_of(circ):
    inv = C.Circuit(circ.n_qubits)
    for ins in reversed(circ.instrs):
        if ins.name == "u3":
            th, ph, la = ins.params
            inv.gate("u3", ins.qubits, (-th, -la, -ph))
        elif ins.name == "cx":
            inv.gate("cx", ins.qubits)
        else:
            raise ValueError("no inverse for " + ins.name)
    return inv


def round_trip(n, depth, seed):
    fwd = C.matching_circuit(n, depth, seed, measure=False)
    rt = C.Circuit(n)
    rt.instrs = fwd.instrs + inverse_of(fwd).instrs
    return rt


def test_inverse_construction_on_the_oracle(oracle):
    n = 12
    p = round_trip(n, 8, 3).to_program()
    _, _, sv, _ = oracle.run(p, prec=64, shots=0, statevector=True)
    want = np.zeros(1 << n, complex)
    want[0] = 1.0
    assert np.abs(sv - want).max() < 1e-12
    # and the forward half alone is far from |0...0>
    fwd = C.matching_circuit(n, 8, 3, measure=False).to_program()
    _, _, sv1, _ = oracle.run(fwd, prec=64, shots=0, statevector=True)
    assert abs(sv1[0]) < 0.5


@pytest.mark.gpu
def test_headline_circuit_round_trip_30q(zc):
    n = 30
    prog = zc.compile(round_trip(n, 40, 7).to_program(), 1)
    be = zc.CudaBackend(n, 64, zc.FLAG_FAST)
    for op in prog.ops:
        if op.kind == zc.OP_UNITARY:
            be.apply_unitary(list(op.qubits), op.data.reshape(1 << len(op.qubits), -1))
        elif op.kind == zc.OP_DIAG:
            be.apply_diagonal(list(op.qubits), op.data)
        elif op.kind == zc.OP_CX:
            be.apply_cx(op.a, op.b)
        else:
            be.apply_swap(op.a, op.b)
    be.finish()
    norm = be.norm_sqr()
    p1 = max(be.prob_one(q) for q in range(n))
    idx = be.sample(1024, 5)
    be.close()
    # fast f64 keeps each amplitude within ~1e-15 per op: the mass that
    # leaves |0...0> over 3,600 gates is far below these bounds
    assert abs(norm - 1.0) < 1e-9, norm
    assert p1 < 1e-12, p1
    assert not np.any(idx), np.unique(idx)[:8]


@pytest.mark.gpu
def test_headline_circuit_fast_vs_exact_30q(zc):
    """The headline circuit itself at its full size: fast f64 against exact
    mode, which reproduces zeno's arithmetic bit for bit (the oracle
    comparisons at every size the oracle can hold). max |d amp| within the
    fast-mode 1e-12 and TVD <= 1e-6, compared in chunks of the two 16 GiB
    states."""
    n = 30
    p = C.matching_circuit(n, 40, 7, measure=False).to_program()
    prog = zc.compile(p, 1)
    fast = zc.run(p, shots=0, precision=64, statevector=True, flags=zc.FLAG_FAST, program=prog).statevector
    exact = zc.run(p, shots=0, precision=64, statevector=True, flags=zc.FLAG_EXACT, program=prog).statevector
    assert fast.shape == exact.shape == (1 << n,)
    d, tvd, chunk = 0.0, 0.0, 1 << 24
    for i in range(0, 1 << n, chunk):
        a, b = fast[i:i + chunk], exact[i:i + chunk]
        d = max(d, float(np.abs(a - b).max()))
        tvd += 0.5 * float(np.abs(np.abs(a) ** 2 - np.abs(b) ** 2).sum())
    assert d < 1e-12, d
    assert tvd < 1e-6, tvd
