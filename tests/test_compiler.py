"""The backend's host compiler (libzeno_cuda zc_compile) against the oracle's
restatement of compiler::compile (src/compiler.rs:118-626): same op kinds,
supports and bit-identical fused matrices at every fusion level 0..6.
Runs on CPU (the compiler needs no GPU)."""

import math

import numpy as np
import pytest

import refmats
from helpers import program_from_json
from test_oracle import _mixed
from zeno_gb300 import circuit as C

pytestmark = []


def _same_ops(zc, oracle, p, fusion):
    mine = zc.compile(p, fusion, swap_perm=False)
    ref = oracle.compile(p, fusion)
    assert mine.dynamic == ref.dynamic
    assert mine.final_measures == ref.final_measures
    assert mine.stats == ref.stats
    a, b = mine.ops, ref.ops
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert x.kind == y.kind
        if x.kind in (0, 1):
            assert x.qubits == y.qubits
            assert np.array_equal(x.data.view(np.float64), y.data.view(np.float64))
        elif x.kind == 2:
            assert (x.a, x.b) == (y.control, y.target)
        elif x.kind in (3, 4):
            assert x.a == y.qubit
        assert x.cond == y.cond


@pytest.mark.parametrize("n", [2, 3, 5, 8])
def test_compiler_matches_oracle(zc, oracle, n):
    for c in (C.random_circuit(n, 12, 100 + n), _mixed(n, 80, 700 + n), C.matching_circuit(n, 6, 5)):
        for fusion in range(7):
            _same_ops(zc, oracle, c.to_program(), fusion)


def test_compiler_examples(zc, oracle, examples):
    for name, d in examples.items():
        p = program_from_json(d)
        for fusion in (0, 1, 5):
            _same_ops(zc, oracle, p, fusion)


def test_swap_stays_a_permutation(zc):
    c = C.Circuit(4)
    c.h(0).swap(3, 1).measure_all()
    ops = zc.compile(c.to_program(), 1).ops
    assert [o.kind for o in ops] == [0, 6]
    assert (ops[1].a, ops[1].b) == (1, 3)


def test_fusion7_support(zc):
    c = C.Circuit(8)
    for q in range(7):
        c.h(q)
    for q in range(6):
        c.cx(q, q + 1)
    p = zc.compile(c.to_program(), 7)
    assert p.stats["max_fused"] == 7 and len(p.ops) == 1
    u = p.ops[0].data.reshape(128, 128)
    assert np.abs(u @ u.conj().T - np.eye(128)).max() < 1e-12


def test_compile_errors(zc):
    c = C.Circuit(2)
    c.gate("cx", [0, 0])
    with pytest.raises(zc.ZenoCudaError, match="duplicate"):
        zc.compile(c.to_program())
    c = C.Circuit(2)
    c.gate("foo", [0])
    with pytest.raises(zc.ZenoCudaError, match="unknown gate"):
        zc.compile(c.to_program())
    c = C.Circuit(2)
    c.gate("rx", [0], [])
    with pytest.raises(zc.ZenoCudaError, match="parameter"):
        zc.compile(c.to_program())
    c = C.Circuit(2)
    c.gate("h", [5])
    with pytest.raises(zc.ZenoCudaError, match="out of range"):
        zc.compile(c.to_program())


def _cancel_case(build, n=3):
    c = C.Circuit(n)
    build(c)
    return c.to_program()


@pytest.mark.parametrize("build, cancelled", [
    (lambda c: c.h(0).h(0), 2),                                    # self-inverse pair
    (lambda c: c.cx(0, 1).x(2).cx(0, 1), 2),                       # a gate on other qubits does not block
    (lambda c: c.cx(0, 1).x(1).cx(0, 1), 0),                       # an overlapping gate does
    (lambda c: c.cx(0, 1).cx(1, 0), 0),                            # same gate, other argument order
    (lambda c: c.swap(0, 1).swap(1, 0), 0),                        # (also for symmetric gates)
    (lambda c: c.x(0).h(0).h(0).x(0), 4),                          # nested pairs unwind
    (lambda c: c.h(0).barrier().h(0), 0),                          # a barrier ends the search
    (lambda c: c.rx(0, 0.3).rx(0, 0.3), 0),                        # gates with parameters never cancel
    (lambda c: c.ccx(0, 1, 2).cz(0, 1).ccx(0, 1, 2), 0),
    (lambda c: c.ccx(0, 1, 2).ccx(0, 1, 2).cz(1, 2).cz(1, 2), 4),
])
def test_cancellation_identities(zc, oracle, build, cancelled):
    """compiler::cancel (src/compiler.rs:215-239): a parameterless
    self-inverse gate cancels against the nearest earlier gate that shares a
    qubit when that gate is the same gate on the same qubits in the same
    order (tests/analytic.rs cancellation identities)."""
    p = _cancel_case(build)
    mine = zc.compile(p, 1, swap_perm=False)
    assert mine.stats["cancelled"] == cancelled
    assert oracle.compile(p, 1).stats["cancelled"] == cancelled
    if cancelled == len(p.instrs):
        assert mine.ops == []
    for fusion in (0, 1, 3):
        _same_ops(zc, oracle, p, fusion)


@pytest.mark.parametrize("build", [
    lambda c: c,                                                   # no instructions at all
    lambda c: c.measure_all(),                                     # measurements only
    lambda c: c.barrier().barrier(),                               # barriers only
    lambda c: c.x(0).barrier().x(0).measure_all(),                 # a barrier between a pair
    lambda c: [c.rz(q, 0.1 * (q + 1)) for q in range(c.n_qubits)] and c,   # one diagonal over every qubit
    lambda c: [c.cz(q, q + 1) for q in range(c.n_qubits - 1)] and c.cp(0, c.n_qubits - 1, 0.7),
])
@pytest.mark.parametrize("n", [1, 12])
def test_degenerate_programs(zc, oracle, build, n):
    """Empty, measure-only and barrier-only programs, and diagonal ladders
    over 12 qubits (wider than the 10-qubit diagonal fusion cap,
    src/compiler.rs:111-114): same ops as the oracle at every fusion level."""
    c = C.Circuit(n)
    try:
        build(c)
    except IndexError:
        pytest.skip("needs two qubits")
    p = c.to_program()
    for fusion in (0, 1, 5):
        _same_ops(zc, oracle, p, fusion)
