"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads `oracle/_build/libzeno_oracle.so` (the C restatement of zeno's scalar
CPU backend, sampler, executor, noise channels, gate library and compiler;
see zeno_oracle.h for the reference file:line map).  Only the tests,
`__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` use it, to
check results and to time the CPU baseline; the shipped library never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libzeno_oracle.so")


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(os.path.join(HERE, f)) for f in ("zeno_oracle.c", "zeno_oracle.h")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


class C64(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class ZoInstr(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("cond_creg", C.c_int32), ("cond_value", C.c_uint64),
        ("name", C.c_char * 8), ("nq", C.c_uint32), ("np", C.c_uint32),
        ("q", C.c_uint32 * 3), ("p", C.c_double * 3), ("clbit", C.c_uint32), ("_pad", C.c_uint32),
    ]


class ZoOp(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("k", C.c_uint32), ("qubits", C.c_uint32 * 12), ("data", C.POINTER(C64)),
        ("control", C.c_uint32), ("target", C.c_uint32), ("qubit", C.c_uint32), ("clbit", C.c_uint32),
        ("has_if", C.c_int32), ("creg_offset", C.c_uint32), ("creg_len", C.c_uint32),
        ("value", C.c_uint64),
    ]


class ZoStats(C.Structure):
    _fields_ = [("input_gates", C.c_uint64), ("cancelled", C.c_uint64), ("output_ops", C.c_uint64),
                ("max_fused", C.c_uint64)]


class ZoNoise(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "depolarizing_1q", "depolarizing_2q", "bit_flip", "phase_flip", "amplitude_damping",
        "readout_flip_0to1", "readout_flip_1to0")]


OP_UNITARY, OP_DIAG, OP_CX, OP_MEASURE, OP_RESET = 0, 1, 2, 3, 4

_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        vp, u32, u64, i32, dbl = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_double
        P = C.POINTER
        L.zo_compile.argtypes = [u32, P(u32), u32, P(ZoInstr), C.c_size_t, u32, u32, P(vp), C.c_char_p,
                                 C.c_size_t]
        L.zo_compile.restype = i32
        L.zo_compiled_free.argtypes = [vp]
        L.zo_compiled_nops.argtypes = [vp]
        L.zo_compiled_nops.restype = C.c_size_t
        L.zo_compiled_op.argtypes = [vp, C.c_size_t]
        L.zo_compiled_op.restype = P(ZoOp)
        L.zo_compiled_dynamic.argtypes = [vp]
        L.zo_compiled_nfinal.argtypes = [vp]
        L.zo_compiled_nfinal.restype = C.c_size_t
        L.zo_compiled_final.argtypes = [vp, C.c_size_t, P(u32), P(u32)]
        L.zo_compiled_stats.argtypes = [vp, P(ZoStats)]
        L.zo_state_new.argtypes = [u32, i32]
        L.zo_state_new.restype = vp
        L.zo_state_free.argtypes = [vp]
        L.zo_set_threads.argtypes = [i32]
        L.zo_get_threads.restype = i32
        L.zo_apply_unitary.argtypes = [vp, P(u32), u32, P(C64)]
        L.zo_apply_diagonal.argtypes = [vp, P(u32), u32, P(C64)]
        L.zo_apply_cx.argtypes = [vp, u32, u32]
        L.zo_prob_one.argtypes = [vp, u32]
        L.zo_prob_one.restype = dbl
        L.zo_measure.argtypes = [vp, u32, dbl]
        L.zo_measure.restype = i32
        L.zo_reset_all.argtypes = [vp]
        L.zo_sample.argtypes = [vp, u64, u64, P(u64)]
        L.zo_statevector.argtypes = [vp, P(C64)]
        L.zo_norm_sqr.argtypes = [vp]
        L.zo_norm_sqr.restype = dbl
        L.zo_load_state.argtypes = [vp, P(C64)]
        L.zo_run.argtypes = [vp, i32, u64, u64, P(ZoNoise), P(u64), P(u64), C.c_size_t, P(C64)]
        L.zo_run.restype = C.c_long
        L.zo_state_bytes.argtypes = [u32, i32]
        L.zo_state_bytes.restype = u64
        L.zo_max_qubits.argtypes = [u64, i32]
        L.zo_max_qubits.restype = u32
        L.zo_refsim_apply.argtypes = [P(C64), u32, P(u32), u32, P(C64)]
        L.zo_gate_build.argtypes = [C.c_char_p, P(dbl), i32, P(i32), P(C64)]
        L.zo_gate_build.restype = i32
        L.zo_splitmix64.argtypes = [u64]
        L.zo_splitmix64.restype = u64
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().zo_set_threads(int(n))


def threads() -> int:
    return int(lib().zo_get_threads())


def _c64_ptr(a: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a, a.ctypes.data_as(C.POINTER(C64))


def _u32_arr(xs: Sequence[int]):
    arr = (C.c_uint32 * max(1, len(xs)))(*xs)
    return arr


def encode_program(p) -> Tuple[C.Array, C.Array, int]:
    ins = (ZoInstr * max(1, len(p.instrs)))()
    for i, x in enumerate(p.instrs):
        z = ins[i]
        z.kind = x.kind
        z.cond_creg = x.cond_creg
        z.cond_value = x.cond_value
        z.name = x.name.encode()[:7]
        z.nq = len(x.qubits) if x.kind == 0 else 1
        z.np = len(x.params)
        for j, q in enumerate(x.qubits[:3]):
            z.q[j] = q
        for j, v in enumerate(x.params[:3]):
            z.p[j] = v
        z.clbit = x.clbit
    cregs = _u32_arr([s for _, s in p.cregs])
    return ins, cregs, len(p.instrs)


class Op:
    """A compiled op (COp, src/compiler.rs:25-55) copied out of the oracle."""

    __slots__ = ("kind", "qubits", "data", "control", "target", "qubit", "clbit", "cond")

    def __init__(self, z: ZoOp):
        self.kind = z.kind
        self.qubits = tuple(z.qubits[i] for i in range(z.k))
        self.data = None
        if z.kind in (OP_UNITARY, OP_DIAG):
            dim = 1 << z.k
            n = dim * dim if z.kind == OP_UNITARY else dim
            raw = np.ctypeslib.as_array(C.cast(z.data, C.POINTER(C.c_double)), shape=(2 * n,))
            self.data = raw.view(np.complex128).copy()
        self.control, self.target = z.control, z.target
        self.qubit, self.clbit = z.qubit, z.clbit
        self.cond = (z.creg_offset, z.creg_len, z.value) if z.has_if else None

    def __repr__(self):
        return "Op(kind=%d, qubits=%s, c=%d, t=%d)" % (self.kind, self.qubits, self.control, self.target)


class Compiled:
    def __init__(self, handle, n_qubits, cregs):
        self._h = handle
        self.n_qubits = n_qubits
        self.cregs = cregs
        L = lib()
        self.ops = [Op(L.zo_compiled_op(handle, i).contents) for i in range(L.zo_compiled_nops(handle))]
        self.dynamic = bool(L.zo_compiled_dynamic(handle))
        q, c = C.c_uint32(), C.c_uint32()
        self.final_measures = []
        for i in range(L.zo_compiled_nfinal(handle)):
            L.zo_compiled_final(handle, i, C.byref(q), C.byref(c))
            self.final_measures.append((q.value, c.value))
        st = ZoStats()
        L.zo_compiled_stats(handle, C.byref(st))
        self.stats = dict(input_gates=st.input_gates, cancelled=st.cancelled, output_ops=st.output_ops,
                          max_fused=st.max_fused)

    def __del__(self):
        try:
            if self._h:
                lib().zo_compiled_free(self._h)
        except Exception:
            pass


class OracleError(RuntimeError):
    pass


def compile(p, fusion_max: int = 1, diag_max: int = 10) -> Compiled:
    """compiler::compile (src/compiler.rs:118-200)."""
    ins, cregs, n = encode_program(p)
    h = C.c_void_p()
    err = C.create_string_buffer(256)
    rc = lib().zo_compile(p.n_qubits, cregs, len(p.cregs), ins, n, fusion_max, diag_max, C.byref(h), err, 256)
    if rc != 0:
        raise OracleError(err.value.decode())
    return Compiled(h, p.n_qubits, list(p.cregs))


def gate_matrix(name: str, params: Sequence[float] = ()) -> Tuple[int, np.ndarray]:
    """gates::build (src/gates.rs:119-188): (kind, matrix or diagonal)."""
    out = np.zeros(64, dtype=np.complex128)
    kind = C.c_int32()
    pa = (C.c_double * 3)(*params)
    ar = lib().zo_gate_build(name.encode(), pa, len(params), C.byref(kind), out.ctypes.data_as(C.POINTER(C64)))
    if ar == 0:
        raise OracleError("unknown gate or wrong parameter count: %s" % name)
    dim = 1 << ar
    return kind.value, (out[: dim * dim].reshape(dim, dim) if kind.value == 0 else out[:dim].copy())


class State:
    """CpuBackend<T> (src/exec.rs:164-225)."""

    def __init__(self, n: int, prec: int = 64):
        self.n, self.prec = n, prec
        self._h = lib().zo_state_new(n, prec)
        if not self._h:
            raise MemoryError("oracle state allocation failed")

    def close(self):
        if self._h:
            lib().zo_state_free(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def apply_unitary(self, qs, mat):
        m, mp = _c64_ptr(np.asarray(mat).reshape(-1))
        lib().zo_apply_unitary(self._h, _u32_arr(qs), len(qs), mp)

    def apply_diagonal(self, qs, d):
        m, mp = _c64_ptr(np.asarray(d).reshape(-1))
        lib().zo_apply_diagonal(self._h, _u32_arr(qs), len(qs), mp)

    def apply_cx(self, c, t):
        lib().zo_apply_cx(self._h, c, t)

    def apply_op(self, op: Op):
        if op.kind == OP_UNITARY:
            self.apply_unitary(op.qubits, op.data)
        elif op.kind == OP_DIAG:
            self.apply_diagonal(op.qubits, op.data)
        elif op.kind == OP_CX:
            self.apply_cx(op.control, op.target)
        else:
            raise ValueError("non-unitary op in a static body")

    def prob_one(self, q) -> float:
        return lib().zo_prob_one(self._h, q)

    def measure(self, q, u) -> bool:
        return bool(lib().zo_measure(self._h, q, u))

    def reset_all(self):
        lib().zo_reset_all(self._h)

    def sample(self, shots: int, seed: int) -> np.ndarray:
        out = np.zeros(max(1, shots), dtype=np.uint64)
        lib().zo_sample(self._h, shots, seed, out.ctypes.data_as(C.POINTER(C.c_uint64)))
        return out[:shots]

    def statevector(self) -> np.ndarray:
        out = np.zeros(1 << self.n, dtype=np.complex128)
        lib().zo_statevector(self._h, out.ctypes.data_as(C.POINTER(C64)))
        return out

    def load(self, amps: np.ndarray):
        a, ap = _c64_ptr(amps)
        lib().zo_load_state(self._h, ap)

    def norm_sqr(self) -> float:
        return lib().zo_norm_sqr(self._h)


def noise_struct(noise) -> Optional[ZoNoise]:
    if noise is None:
        return None
    z = ZoNoise()
    for f, _ in ZoNoise._fields_:
        setattr(z, f, float(getattr(noise, f)))
    return z


def run(p, prec: int = 64, shots: int = 1024, seed: int = 0, fusion: int = 1, noise=None,
        statevector: bool = False):
    """zeno::run_program (src/lib.rs:224-250 → src/exec.rs:347-396).

    Returns (counts {key: n}, raw {clbit word: n}, statevector or None, Compiled).
    """
    noisy = noise is not None and any(getattr(noise, f) != 0.0 for f, _ in ZoNoise._fields_)
    c = compile(p, 0 if noisy else fusion)
    cap = max(16, shots + 1)
    keys = np.zeros(cap, dtype=np.uint64)
    counts = np.zeros(cap, dtype=np.uint64)
    sv = np.zeros(1 << p.n_qubits, dtype=np.complex128) if statevector else None
    nz = noise_struct(noise) if noisy else None
    m = lib().zo_run(c._h, prec, shots, seed, C.byref(nz) if nz is not None else None,
                     keys.ctypes.data_as(C.POINTER(C.c_uint64)), counts.ctypes.data_as(C.POINTER(C.c_uint64)),
                     cap, sv.ctypes.data_as(C.POINTER(C64)) if sv is not None else None)
    if m < 0:
        raise OracleError("run rejected (statevector with a dynamic or noisy circuit)")
    raw = {int(keys[i]): int(counts[i]) for i in range(m)}
    fmt: Dict[str, int] = {}
    for k, v in raw.items():
        key = format_key(k, p.cregs)
        fmt[key] = fmt.get(key, 0) + v
    return fmt, raw, sv, c


def format_key(clbits: int, cregs) -> str:
    """Counts key, qiskit convention (src/exec.rs:235-253)."""
    if not cregs:
        return ""
    parts, off = [], 0
    for _, size in cregs:
        mask = (1 << 64) - 1 if size >= 64 else (1 << size) - 1
        parts.append(format((clbits >> off) & mask, "b").rjust(size, "0"))
        off += size
    return " ".join(reversed(parts))


def refsim_apply(amps: np.ndarray, n: int, qs: Sequence[int], mat: np.ndarray) -> None:
    """Independent dense apply (tests/reference.rs:69-116), in place."""
    assert amps.dtype == np.complex128 and amps.flags.c_contiguous
    m, mp = _c64_ptr(np.asarray(mat).reshape(-1))
    lib().zo_refsim_apply(amps.ctypes.data_as(C.POINTER(C64)), n, _u32_arr(qs), len(qs), mp)


def state_bytes(n: int, prec: int) -> int:
    return int(lib().zo_state_bytes(n, prec))


def max_qubits(budget: int, prec: int) -> int:
    return int(lib().zo_max_qubits(budget, prec))
