"""Shared test utilities: seeded random states, golden-program loading."""

import math

import numpy as np

from zeno_gb300 import circuit as C


class Sm64:
    """splitmix64 test stream (the reference's test RNG, src/state.rs:1304-1334)."""

    M = (1 << 64) - 1

    def __init__(self, seed):
        self.x = seed & self.M

    def next(self):
        self.x = (self.x + 0x9E3779B97F4A7C15) & self.M
        z = self.x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.M
        return z ^ (z >> 31)

    def sym(self):
        return float(self.next() >> 11) / float(1 << 52) - 1.0

    def uniform(self):
        return float(self.next() >> 11) / float(1 << 53)

    def angle(self):
        return (self.uniform() * 2.0 - 1.0) * math.pi

    def below(self, n):
        return self.next() % n


def rand_state(n, seed, normalize=False):
    """Random complex vector (numpy generator; amplitudes in [-1, 1))."""
    g = np.random.default_rng(seed)
    a = g.uniform(-1, 1, 1 << n) + 1j * g.uniform(-1, 1, 1 << n)
    if normalize:
        a /= np.linalg.norm(a)
    return a.astype(np.complex128)


def rand_matrix(dim, seed):
    g = np.random.default_rng(seed)
    return (g.uniform(-1, 1, (dim, dim)) + 1j * g.uniform(-1, 1, (dim, dim))).astype(np.complex128)


def as_precision(a, prec):
    """Round a c128 vector to the state precision (what the backend stores)."""
    if prec == 32:
        return (a.real.astype(np.float32).astype(np.float64) + 1j * a.imag.astype(np.float32).astype(np.float64))
    return a


def program_from_json(d):
    p = C.Program(d["n_qubits"], [tuple(c) for c in d["cregs"]], [])
    for i in d["instrs"]:
        cond = i.get("cond")
        p.instrs.append(C.Instr(i["kind"], i.get("name", ""), tuple(i.get("qubits", ())),
                                tuple(i.get("params", ())), i.get("clbit", 0),
                                cond[0] if cond else -1, cond[1] if cond else 0))
    return p


def bits_equal(a, b):
    """Exact equality of two c128 arrays (values; -0.0 == 0.0)."""
    return np.array_equal(a.real, b.real) and np.array_equal(a.imag, b.imag)


def max_delta(a, b):
    return float(np.max(np.abs(a - b))) if len(a) else 0.0


def supports(n, k):
    out = []
    for m in range(1 << n):
        if bin(m).count("1") == k:
            out.append(tuple(b for b in range(n) if (m >> b) & 1))
    return out
