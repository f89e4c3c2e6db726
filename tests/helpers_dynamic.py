"""Seeded dynamic circuits: mid-circuit measurements into 1-bit registers,
operations conditioned on them, resets, and final measurements."""

import math

import numpy as np

from zeno_gb300 import circuit as C


def dynamic_program(n, layers, seed):
    """Layers of u3 on every qubit + CX on neighbour pairs; after each layer,
    measure one qubit into its own 1-bit register, apply a gate conditioned
    on that bit (x, u3 or z on another qubit), reset the measured qubit.
    Final measurement of every qubit into register f."""
    rng = np.random.default_rng(seed)
    cregs = [("m%d" % i, 1) for i in range(layers)] + [("f", n)]
    p = C.Program(n, cregs, [])
    I = C.Instr
    for layer in range(layers):
        for q in range(n):
            p.instrs.append(I(C.I_GATE, "u3", (q,), tuple(float(x) for x in rng.uniform(0, 2 * math.pi, 3))))
        for q in range(layer % 2, n - 1, 2):
            p.instrs.append(I(C.I_GATE, "cx", (q, q + 1)))
        mq = int(rng.integers(n))
        p.instrs.append(I(C.I_MEASURE, qubits=(mq,), clbit=layer))
        tq = (mq + 1 + int(rng.integers(n - 1))) % n
        kind = layer % 3
        if kind == 0:
            p.instrs.append(I(C.I_GATE, "x", (tq,), (), 0, layer, 1))
        elif kind == 1:
            p.instrs.append(I(C.I_GATE, "u3", (tq,), (0.7, 0.2, 1.1), 0, layer, 1))
        else:
            p.instrs.append(I(C.I_GATE, "z", (tq,), (), 0, layer, 0))
        p.instrs.append(I(C.I_RESET, qubits=(mq,)))
    for q in range(n):
        p.instrs.append(I(C.I_MEASURE, qubits=(q,), clbit=layers + q))
    return p
