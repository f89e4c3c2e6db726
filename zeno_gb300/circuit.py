"""Circuit IR, builder and seeded workload generators.

The IR mirrors zeno's `ir::Program` (src/ir.rs:36-63): registers plus a flat
instruction list in which a gate's qubits are in argument order and bit `q`
of a basis index is qubit `q` (little-endian).  `Circuit` mirrors the
builder of src/circuit.rs:18-134.

Generators:
  * `random_circuit`    — zeno's own brickwork (src/circuit.rs:152-174):
                          u3 on every qubit, then an alternating CX ladder.
  * `matching_circuit`  — u3 on every qubit with angles U[0, 2pi), then CX on
                          a seeded random perfect matching with random
                          orientation (the 20q/30q/33q/16q workloads).
  * `qft_circuit`       — |x> prepared by X gates, H + cp(pi/2^k) for every
                          pair (the order of src/circuit.rs:138-148), then
                          the final SWAP network.
  * `mixed_circuit`     — gates per slot from {H,S,T,RX/RY/RZ,CX,CZ,SWAP}
                          with probabilities {.15,.1,.1,.3,.25,.05,.05}.
All randomness comes from xoshiro256++ seeded like rand_xoshiro's
`seed_from_u64`, with rand 0.8's f64 and integer-range draws.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

from .rng import Xoshiro256pp

I_GATE, I_MEASURE, I_RESET, I_BARRIER = 0, 1, 2, 3

TAU = 2.0 * math.pi

# name -> (arity, n_params); src/gates.rs:101-115
NATIVE_GATES = {
    "id": (1, 0), "u0": (1, 0), "x": (1, 0), "y": (1, 0), "z": (1, 0), "h": (1, 0),
    "s": (1, 0), "sdg": (1, 0), "t": (1, 0), "tdg": (1, 0), "sx": (1, 0), "sxdg": (1, 0),
    "rx": (1, 1), "ry": (1, 1), "rz": (1, 1), "u1": (1, 1), "p": (1, 1), "u2": (1, 2),
    "u3": (1, 3), "u": (1, 3), "cx": (2, 0), "cy": (2, 0), "cz": (2, 0), "ch": (2, 0),
    "swap": (2, 0), "cp": (2, 1), "cu1": (2, 1), "crx": (2, 1), "cry": (2, 1), "crz": (2, 1),
    "rxx": (2, 1), "rzz": (2, 1), "cu3": (2, 3), "ccx": (3, 0), "cswap": (3, 0),
}


@dataclass
class Instr:
    """One program instruction (src/ir.rs:36-52). `cond_creg >= 0` wraps it
    in `if (creg == cond_value)`."""

    kind: int
    name: str = ""
    qubits: Tuple[int, ...] = ()
    params: Tuple[float, ...] = ()
    clbit: int = 0
    cond_creg: int = -1
    cond_value: int = 0


@dataclass
class Program:
    """Registers plus a flat instruction list (src/ir.rs:59-83)."""

    n_qubits: int
    cregs: List[Tuple[str, int]] = field(default_factory=list)
    instrs: List[Instr] = field(default_factory=list)

    @property
    def n_clbits(self) -> int:
        return sum(s for _, s in self.cregs)

    def creg_offset(self, idx: int) -> int:
        return sum(s for _, s in self.cregs[:idx])


class Circuit:
    """Builder with one `q` register and one `c` register (src/circuit.rs)."""

    def __init__(self, n_qubits: int):
        self.n_qubits = int(n_qubits)
        self.instrs: List[Instr] = []

    def gate(self, name: str, qubits: Sequence[int], params: Sequence[float] = ()) -> "Circuit":
        self.instrs.append(Instr(I_GATE, name, tuple(int(q) for q in qubits),
                                 tuple(float(p) for p in params)))
        return self

    def __getattr__(self, name):
        if name in NATIVE_GATES:
            arity, npar = NATIVE_GATES[name]

            def f(*args):
                qs, ps = args[:arity], args[arity:]
                return self.gate("u3" if name == "u" else name, qs, ps)

            return f
        raise AttributeError(name)

    def measure(self, qubit: int, clbit: int) -> "Circuit":
        self.instrs.append(Instr(I_MEASURE, qubits=(int(qubit),), clbit=int(clbit)))
        return self

    def measure_all(self) -> "Circuit":
        for q in range(self.n_qubits):
            self.measure(q, q)
        return self

    def reset(self, qubit: int) -> "Circuit":
        self.instrs.append(Instr(I_RESET, qubits=(int(qubit),)))
        return self

    def barrier(self) -> "Circuit":
        self.instrs.append(Instr(I_BARRIER, qubits=tuple(range(self.n_qubits))))
        return self

    def to_program(self) -> Program:
        return Program(self.n_qubits, [("c", self.n_qubits)], list(self.instrs))


def input_gate_count(p: Program) -> int:
    """`Stats::input_gates` (src/compiler.rs:202-211)."""
    return sum(1 for i in p.instrs if i.kind == I_GATE)


# --------------------------------------------------------------- generators


def random_circuit(n: int, depth: int, seed: int) -> Circuit:
    """zeno's `random_circuit` brickwork (src/circuit.rs:152-174)."""
    rng = Xoshiro256pp(seed)
    c = Circuit(n)
    for layer in range(depth):
        for q in range(n):
            c.u(q, rng.f64() * TAU, rng.f64() * TAU, rng.f64() * TAU)
        q = layer % 2
        while q + 1 < n:
            c.cx(q, q + 1)
            q += 2
    return c


def matching_circuit(n: int, depth: int, seed: int, measure: bool = True) -> Circuit:
    """u3 layer + CX on a random perfect matching, `depth` times.

    Per layer: for q = 0..n-1 draw theta, phi, lambda = 2pi*U[0,1) (in that
    order); then Fisher-Yates shuffle of 0..n-1 (i from n-1 down to 1, j =
    range(0, i+1)); pairs (perm[2j], perm[2j+1]); each pair's orientation is
    flipped when a further U[0,1) draw is < 0.5.  An odd qubit out is idle.
    """
    rng = Xoshiro256pp(seed)
    c = Circuit(n)
    for _ in range(depth):
        for q in range(n):
            th, ph, la = rng.f64() * TAU, rng.f64() * TAU, rng.f64() * TAU
            c.u(q, th, ph, la)
        perm = list(range(n))
        for i in range(n - 1, 0, -1):
            j = rng.range(0, i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        for k in range(n // 2):
            a, b = perm[2 * k], perm[2 * k + 1]
            if rng.f64() < 0.5:
                a, b = b, a
            c.cx(a, b)
    if measure:
        c.measure_all()
    return c


def qft_circuit(n: int, seed: int, swaps: bool = True, measure: bool = True) -> Tuple[Circuit, int]:
    """QFT of a seeded basis state |x>; returns (circuit, x).

    x = range(0, 2^n) from the seeded stream; X on every set bit of x; then
    for i = n-1..0: H(i), cp(pi/2^(i-j)) on (j, i) for j = i-1..0 (the
    ladder of src/circuit.rs:138-148); then SWAP(k, n-1-k) for k < n/2.
    """
    rng = Xoshiro256pp(seed)
    x = rng.range(0, 1 << n)
    c = Circuit(n)
    for q in range(n):
        if (x >> q) & 1:
            c.x(q)
    for i in range(n - 1, -1, -1):
        c.h(i)
        for j in range(i - 1, -1, -1):
            c.cp(j, i, math.pi / float(1 << (i - j)))
    if swaps:
        for k in range(n // 2):
            c.swap(k, n - 1 - k)
    if measure:
        c.measure_all()
    return c, x


_MIX = [("h", 0.15), ("s", 0.10), ("t", 0.10), ("rot", 0.30), ("cx", 0.25), ("cz", 0.05), ("swap", 0.05)]


def mixed_circuit(n: int, depth: int, seed: int, measure: bool = True) -> Circuit:
    """Random gate mix, `depth` layers.

    Per layer: shuffle the qubits (as in `matching_circuit`) and walk the
    order; each slot draws U[0,1) against the cumulative table
    H .15, S .10, T .10, RX/RY/RZ .30 (then range(0,3) picks the axis and
    2pi*U[0,1) the angle), CX .25, CZ .05, SWAP .05.  A two-qubit pick takes
    the next qubit of the order as its second argument; with none left the
    slot becomes H.
    """
    rng = Xoshiro256pp(seed)
    c = Circuit(n)
    for _ in range(depth):
        perm = list(range(n))
        for i in range(n - 1, 0, -1):
            j = rng.range(0, i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        pos = 0
        while pos < n:
            u = rng.f64()
            acc, kind = 0.0, _MIX[-1][0]
            for name, p in _MIX:
                acc += p
                if u < acc:
                    kind = name
                    break
            q = perm[pos]
            if kind in ("cx", "cz", "swap"):
                if pos + 1 < n:
                    c.gate(kind, (q, perm[pos + 1]))
                    pos += 2
                    continue
                kind = "h"
            if kind == "rot":
                axis = ("rx", "ry", "rz")[rng.range(0, 3)]
                c.gate(axis, (q,), (rng.f64() * TAU,))
            else:
                c.gate(kind, (q,))
            pos += 1
    if measure:
        c.measure_all()
    return c


def format_key(clbits: int, cregs: Sequence[Tuple[str, int]]) -> str:
    """Counts key, qiskit convention (src/exec.rs:235-253)."""
    if not cregs:
        return ""
    parts, off = [], 0
    for _, size in cregs:
        mask = (1 << 64) - 1 if size >= 64 else (1 << size) - 1
        parts.append(format((clbits >> off) & mask, "b").rjust(size, "0"))
        off += size
    return " ".join(reversed(parts))
