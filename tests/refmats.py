"""Hand-coded dense gate matrices from the standard definitions (qiskit
U(theta, phi, lambda) convention; controls first = low bits of the local
index), independent of both the oracle's and the backend's gate tables —
the role of `ref_gate` in the reference's tests/reference.rs:131-294 —
plus a numpy dense simulator (the reference's `RefSim`, :69-116)."""

import cmath
import math

import numpy as np


def eip(t):
    return cmath.exp(1j * t)


def dmat(d):
    return np.diag(np.array(d, dtype=np.complex128))


def ctrl1(u):
    m = np.zeros((4, 4), dtype=np.complex128)
    m[0, 0] = 1
    m[2, 2] = 1
    for to in range(2):
        for ti in range(2):
            m[1 + 2 * to, 1 + 2 * ti] = u[to, ti]
    return m


def u3m(t, p, l):
    ct, st = math.cos(t / 2), math.sin(t / 2)
    return np.array([[ct, -eip(l) * st], [eip(p) * st, eip(p + l) * ct]], dtype=np.complex128)


def rxm(t):
    ct, st = math.cos(t / 2), math.sin(t / 2)
    return np.array([[ct, -1j * st], [-1j * st, ct]], dtype=np.complex128)


def rym(t):
    ct, st = math.cos(t / 2), math.sin(t / 2)
    return np.array([[ct, -st], [st, ct]], dtype=np.complex128)


def rzm(t):
    return dmat([eip(-t / 2), eip(t / 2)])


def perm_matrix(dim, f):
    m = np.zeros((dim, dim), dtype=np.complex128)
    for col in range(dim):
        m[f(col), col] = 1
    return m


def ref_gate(name, p=()):
    sq = 1 / math.sqrt(2)
    H = np.array([[sq, sq], [sq, -sq]], dtype=np.complex128)
    Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    if name in ("id", "u0"):
        return np.eye(2, dtype=np.complex128)
    table = {
        "x": lambda: np.array([[0, 1], [1, 0]], dtype=np.complex128),
        "y": lambda: Y,
        "z": lambda: dmat([1, -1]),
        "h": lambda: H,
        "s": lambda: dmat([1, 1j]),
        "sdg": lambda: dmat([1, -1j]),
        "t": lambda: dmat([1, eip(math.pi / 4)]),
        "tdg": lambda: dmat([1, eip(-math.pi / 4)]),
        "sx": lambda: np.array([[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]]),
        "sxdg": lambda: np.array([[0.5 - 0.5j, 0.5 + 0.5j], [0.5 + 0.5j, 0.5 - 0.5j]]),
        "rx": lambda: rxm(p[0]),
        "ry": lambda: rym(p[0]),
        "rz": lambda: rzm(p[0]),
        "u1": lambda: dmat([1, eip(p[0])]),
        "p": lambda: dmat([1, eip(p[0])]),
        "u2": lambda: u3m(math.pi / 2, p[0], p[1]),
        "u3": lambda: u3m(p[0], p[1], p[2]),
        "u": lambda: u3m(p[0], p[1], p[2]),
        "cx": lambda: perm_matrix(4, lambda c: (c & 1) | ((((c >> 1) & 1) ^ (c & 1)) << 1)),
        "cy": lambda: ctrl1(Y),
        "cz": lambda: dmat([1, 1, 1, -1]),
        "ch": lambda: ctrl1(H),
        "swap": lambda: perm_matrix(4, lambda c: ((c & 1) << 1) | ((c >> 1) & 1)),
        "cp": lambda: dmat([1, 1, 1, eip(p[0])]),
        "cu1": lambda: dmat([1, 1, 1, eip(p[0])]),
        "crx": lambda: ctrl1(rxm(p[0])),
        "cry": lambda: ctrl1(rym(p[0])),
        "crz": lambda: ctrl1(rzm(p[0])),
        "cu3": lambda: ctrl1(u3m(p[0], p[1], p[2])),
        "rxx": lambda: math.cos(p[0] / 2) * np.eye(4) - 1j * math.sin(p[0] / 2) * np.fliplr(np.eye(4)),
        "rzz": lambda: dmat([eip(-p[0] / 2), eip(p[0] / 2), eip(p[0] / 2), eip(-p[0] / 2)]),
        "ccx": lambda: perm_matrix(8, lambda c: c ^ 4 if (c & 3) == 3 else c),
        "cswap": lambda: perm_matrix(8, lambda c: (1 | (((c >> 2) & 1) << 1) | (((c >> 1) & 1) << 2))
                                     if c & 1 else c),
    }
    return np.asarray(table[name](), dtype=np.complex128)


NATIVE = [
    ("id", 1, 0), ("u0", 1, 0), ("x", 1, 0), ("y", 1, 0), ("z", 1, 0), ("h", 1, 0), ("s", 1, 0),
    ("sdg", 1, 0), ("t", 1, 0), ("tdg", 1, 0), ("sx", 1, 0), ("sxdg", 1, 0), ("rx", 1, 1), ("ry", 1, 1),
    ("rz", 1, 1), ("u1", 1, 1), ("p", 1, 1), ("u2", 1, 2), ("u3", 1, 3), ("u", 1, 3), ("cx", 2, 0),
    ("cy", 2, 0), ("cz", 2, 0), ("ch", 2, 0), ("swap", 2, 0), ("cp", 2, 1), ("cu1", 2, 1), ("crx", 2, 1),
    ("cry", 2, 1), ("crz", 2, 1), ("rxx", 2, 1), ("rzz", 2, 1), ("cu3", 2, 3), ("ccx", 3, 0), ("cswap", 3, 0),
]


def apply_dense(amps, n, qs, mat):
    """Apply `mat` (argument order: bit b of the local index is qs[b])."""
    k = len(qs)
    t = amps.reshape([2] * n)  # axis a <-> qubit n-1-a
    axes = [n - 1 - q for q in reversed(qs)]  # local index bits high..low
    m = mat.reshape([2] * (2 * k))
    t = np.tensordot(m, t, axes=(list(range(k, 2 * k)), axes))
    t = np.moveaxis(t, list(range(k)), axes)
    return np.ascontiguousarray(t).reshape(-1)


def simulate(p):
    """Dense replay of every gate of a program (measure / barrier ignored)."""
    n = p.n_qubits
    a = np.zeros(1 << n, dtype=np.complex128)
    a[0] = 1
    for ins in p.instrs:
        if ins.kind == 0:
            a = apply_dense(a, n, list(ins.qubits), ref_gate(ins.name, ins.params))
    return a
