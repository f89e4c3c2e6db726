"""ctypes binding of libzeno_cuda.so (include/zeno_cuda.h).

`CudaBackend` mirrors zeno's `exec::Backend` trait (src/exec.rs:134-162)
method for method; `compile` and `run` mirror `compiler::compile` and
`zeno::run_program` (src/lib.rs:224-250). Every call goes through the C ABI
into the sm_103a kernels; there is no CPU fallback — a missing library or a
missing GPU raises.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field, fields
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import circuit as _circ

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libzeno_cuda.so")

ZC_OK, ZC_ERR_INVALID, ZC_ERR_MEMORY, ZC_ERR_CUDA, ZC_ERR_UNSUPPORTED = 0, 1, 2, 3, 4
FLAG_EXACT, FLAG_FAST, FLAG_NO_SWEEPS, FLAG_FORCE_SWEEPS, FLAG_PER_SHOT, FLAG_TENSOR = 0, 1, 2, 4, 8, 16
OP_UNITARY, OP_DIAG, OP_CX, OP_MEASURE, OP_RESET, OP_SWAP = 0, 1, 2, 3, 4, 6

# Every entry point the header declares; the CPU test suite checks exports.
EXPORTS = (
    "zc_create", "zc_create_ex", "zc_destroy", "zc_name", "zc_apply_unitary", "zc_apply_diagonal",
    "zc_apply_cx", "zc_apply_swap", "zc_prob_one", "zc_measure", "zc_reset_all", "zc_sample",
    "zc_statevector", "zc_norm_sqr", "zc_finish", "zc_last_error", "zc_device_budget", "zc_device_memory", "zc_state_bytes",
    "zc_max_qubits", "zc_load_state", "zc_get_stream", "zc_get_counters", "zc_compile", "zc_program_free",
    "zc_program_get_info", "zc_program_get_op", "zc_program_get_final", "zc_run", "zc_profile",
    "zc_profile_read", "zc_sample_noalloc", "zc_set_sweep_shape", "zc_device_info", "zc_measure_arith_peaks",
)


class DeviceC(C.Structure):
    _fields_ = [("name", C.c_char * 64), ("sms", C.c_uint32), ("cc_major", C.c_uint32), ("cc_minor", C.c_uint32),
                ("_pad", C.c_uint32), ("hbm_bytes", C.c_uint64), ("free_bytes", C.c_uint64),
                ("l2_bytes", C.c_uint64)]


class ArithPeaksC(C.Structure):
    _fields_ = [("fp64_fma_per_s", C.c_double), ("fp32_fma_per_s", C.c_double), ("sms", C.c_uint32),
                ("_pad", C.c_uint32)]


class ZenoCudaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class Counters(C.Structure):
    _fields_ = [("ops", C.c_uint64), ("launches", C.c_uint64), ("sweeps", C.c_uint64), ("bytes_moved", C.c_uint64),
                ("micro_ops", C.c_uint64 * 8)]

# Sweep micro-op kinds (zc_counters.micro_ops index).
MICRO_OP_KINDS = {1: "complex", 2: "diag1", 3: "diag_table", 4: "cx", 5: "swap", 6: "real", 7: "rotation"}


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 24), ("launches", C.c_uint64), ("ms", C.c_double), ("bytes", C.c_double)]


class Instr(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("cond_creg", C.c_int32), ("cond_value", C.c_uint64), ("name", C.c_char * 8),
        ("nq", C.c_uint32), ("np", C.c_uint32), ("q", C.c_uint32 * 3), ("p", C.c_double * 3),
        ("clbit", C.c_uint32), ("_pad", C.c_uint32),
    ]


class CompileOptions(C.Structure):
    _fields_ = [("fusion_max", C.c_uint32), ("diag_max", C.c_uint32), ("swap_perm", C.c_uint32)]


class OpView(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("k", C.c_uint32), ("qubits", C.c_uint32 * 12), ("data", C.POINTER(C.c_double)),
        ("a", C.c_uint32), ("b", C.c_uint32), ("has_if", C.c_int32), ("creg_offset", C.c_uint32),
        ("creg_len", C.c_uint32), ("value", C.c_uint64),
    ]


class ProgramInfo(C.Structure):
    _fields_ = [
        ("n_qubits", C.c_uint32), ("n_clbits", C.c_uint32), ("nops", C.c_uint64), ("nfinal", C.c_uint64),
        ("dynamic", C.c_int32), ("input_gates", C.c_uint64), ("cancelled", C.c_uint64),
        ("output_ops", C.c_uint64), ("max_fused", C.c_uint64),
    ]


class NoiseC(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "depolarizing_1q", "depolarizing_2q", "bit_flip", "phase_flip", "amplitude_damping",
        "readout_flip_0to1", "readout_flip_1to0")]


class RunOptions(C.Structure):
    _fields_ = [("precision_bits", C.c_int), ("flags", C.c_uint32), ("shots", C.c_uint64), ("seed", C.c_uint64),
                ("noise", C.POINTER(NoiseC)), ("mem_fraction", C.c_double), ("sweep_high", C.c_uint32),
                ("_pad", C.c_uint32)]


class RunResultC(C.Structure):
    _fields_ = [("precision_bits", C.c_int), ("batched", C.c_int), ("n_keys", C.c_uint64), ("sim_seconds", C.c_double),
                ("launches", C.c_uint64), ("sweeps", C.c_uint64), ("bytes_moved", C.c_uint64),
                ("notices", C.c_char * 512)]


@dataclass
class NoiseModel:
    """NoiseModel (src/noise.rs:39-47): per-gate and readout probabilities."""

    depolarizing_1q: float = 0.0
    depolarizing_2q: float = 0.0
    bit_flip: float = 0.0
    phase_flip: float = 0.0
    amplitude_damping: float = 0.0
    readout_flip_0to1: float = 0.0
    readout_flip_1to0: float = 0.0

    def is_trivial(self) -> bool:
        return all(getattr(self, f.name) == 0.0 for f in fields(self))

    def validate(self) -> None:
        for f in fields(self):
            v = getattr(self, f.name)
            if not (0.0 <= v <= 1.0):
                raise ValueError("invalid noise model: %s = %r is not a probability in [0, 1]" % (f.name, v))


_lib = None


def load() -> C.CDLL:
    """Load the in-tree library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ZenoCudaError(ZC_ERR_UNSUPPORTED,
                            "libzeno_cuda.so is not built (run zeno_gb300.build.build() or __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    vp, u32, u64, i32, dbl, P = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_double, C.POINTER
    sig = {
        "zc_create": ([u32, i32, P(vp)], i32),
        "zc_create_ex": ([u32, i32, u32, P(vp)], i32),
        "zc_destroy": ([vp], None),
        "zc_name": ([vp], C.c_char_p),
        "zc_apply_unitary": ([vp, P(u32), u32, P(dbl)], i32),
        "zc_apply_diagonal": ([vp, P(u32), u32, P(dbl)], i32),
        "zc_apply_cx": ([vp, u32, u32], i32),
        "zc_apply_swap": ([vp, u32, u32], i32),
        "zc_prob_one": ([vp, u32, P(dbl)], i32),
        "zc_measure": ([vp, u32, dbl, P(i32)], i32),
        "zc_reset_all": ([vp], i32),
        "zc_sample": ([vp, u64, u64, P(u64)], i32),
        "zc_statevector": ([vp, P(dbl)], i32),
        "zc_norm_sqr": ([vp, P(dbl)], i32),
        "zc_finish": ([vp], i32),
        "zc_last_error": ([], C.c_char_p),
        "zc_device_budget": ([dbl, P(u64)], i32),
        "zc_device_memory": ([P(u64)], i32),
        "zc_state_bytes": ([u32, i32], u64),
        "zc_max_qubits": ([u64, i32], u32),
        "zc_load_state": ([vp, P(dbl)], i32),
        "zc_get_stream": ([vp, P(vp)], i32),
        "zc_get_counters": ([vp, P(Counters)], i32),
        "zc_compile": ([u32, P(u32), u32, P(Instr), C.c_size_t, P(CompileOptions), P(vp)], i32),
        "zc_program_free": ([vp], None),
        "zc_program_get_info": ([vp, P(ProgramInfo)], i32),
        "zc_program_get_op": ([vp, C.c_size_t, P(OpView)], i32),
        "zc_program_get_final": ([vp, C.c_size_t, P(u32), P(u32)], i32),
        "zc_run": ([vp, P(RunOptions), P(RunResultC), P(u64), P(u64), C.c_size_t, P(dbl)], i32),
        "zc_profile": ([vp, i32], i32),
        "zc_sample_noalloc": ([vp, u64, u64, P(u64)], i32),
        "zc_profile_read": ([vp, P(KernelStat), i32, P(i32)], i32),
        "zc_set_sweep_shape": ([vp, u32], i32),
        "zc_device_info": ([P(DeviceC)], i32),
        "zc_measure_arith_peaks": ([P(ArithPeaksC)], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != ZC_OK:
        raise ZenoCudaError(rc, load().zc_last_error().decode(errors="replace"))


def _u32(xs: Sequence[int]):
    return (C.c_uint32 * max(1, len(xs)))(*[int(x) for x in xs])


def _c64(a) -> Tuple[np.ndarray, "C.POINTER(C.c_double)"]:
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.complex128).reshape(-1))
    return arr, arr.ctypes.data_as(C.POINTER(C.c_double))


class CudaBackend:
    """`Backend` on one GB300 (src/exec.rs:134-162). precision 32 or 64."""

    def __init__(self, n_qubits: int, precision: int = 64, flags: int = FLAG_EXACT):
        self.n = int(n_qubits)
        self.precision = int(precision)
        L = load()
        h = C.c_void_p()
        _check(L.zc_create_ex(self.n, self.precision, flags, C.byref(h)))
        self._h = h

    # --- trait methods
    def name(self) -> str:
        return load().zc_name(self._h).decode()

    def apply_unitary(self, qs: Sequence[int], mat) -> None:
        m, mp = _c64(mat)
        _check(load().zc_apply_unitary(self._h, _u32(qs), len(qs), mp))

    def apply_diagonal(self, qs: Sequence[int], d) -> None:
        m, mp = _c64(d)
        _check(load().zc_apply_diagonal(self._h, _u32(qs), len(qs), mp))

    def apply_cx(self, control: int, target: int) -> None:
        _check(load().zc_apply_cx(self._h, control, target))

    def apply_swap(self, a: int, b: int) -> None:
        _check(load().zc_apply_swap(self._h, a, b))

    def prob_one(self, q: int) -> float:
        out = C.c_double()
        _check(load().zc_prob_one(self._h, q, C.byref(out)))
        return out.value

    def measure(self, q: int, u: float) -> bool:
        out = C.c_int()
        _check(load().zc_measure(self._h, q, float(u), C.byref(out)))
        return bool(out.value)

    def reset_all(self) -> None:
        _check(load().zc_reset_all(self._h))

    def sample(self, shots: int, seed: int) -> np.ndarray:
        out = np.zeros(max(1, shots), dtype=np.uint64)
        _check(load().zc_sample(self._h, shots, seed, out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out[:shots]

    def sample_noalloc(self, shots: int, seed: int) -> np.ndarray:
        """`sample` through the entry point that allocates nothing (for callers
        that cannot allocate device memory at sampling time); flush first."""
        out = np.zeros(max(1, shots), dtype=np.uint64)
        _check(load().zc_sample_noalloc(self._h, shots, seed, out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out[:shots]

    def statevector(self) -> np.ndarray:
        out = np.zeros(1 << self.n, dtype=np.complex128)
        _check(load().zc_statevector(self._h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def norm_sqr(self) -> float:
        out = C.c_double()
        _check(load().zc_norm_sqr(self._h, C.byref(out)))
        return out.value

    def finish(self) -> None:
        _check(load().zc_finish(self._h))

    # --- harness helpers
    def load_state(self, amps) -> None:
        a, ap = _c64(amps)
        assert a.size == 1 << self.n
        _check(load().zc_load_state(self._h, ap))

    def stream(self) -> int:
        s = C.c_void_p()
        _check(load().zc_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def counters(self) -> Dict[str, int]:
        c = Counters()
        _check(load().zc_get_counters(self._h, C.byref(c)))
        out = {f: getattr(c, f) for f, _ in Counters._fields_ if f != "micro_ops"}
        out["micro_ops"] = {name: int(c.micro_ops[k]) for k, name in MICRO_OP_KINDS.items()}
        return out

    def profile(self, enable: bool = True) -> None:
        """Start (and clear) or stop per-launch CUDA-event recording."""
        _check(load().zc_profile(self._h, 1 if enable else 0))

    def set_sweep_shape(self, max_high: int) -> None:
        """At most `max_high` qubits above the row per sweep tile (0: automatic)."""
        _check(load().zc_set_sweep_shape(self._h, max_high))

    def profile_read(self) -> Dict[str, Dict[str, float]]:
        """Per kernel class: launches, total ms, algorithmic bytes (flushes and syncs)."""
        arr = (KernelStat * 32)()
        n = C.c_int()
        _check(load().zc_profile_read(self._h, arr, 32, C.byref(n)))
        return {arr[i].name.decode(): {"launches": arr[i].launches, "ms": arr[i].ms, "bytes": arr[i].bytes}
                for i in range(min(n.value, 32))}

    def close(self) -> None:
        if getattr(self, "_h", None):
            load().zc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


# ------------------------------------------------------------------ pipeline


@dataclass
class Op:
    kind: int
    qubits: Tuple[int, ...]
    data: Optional[np.ndarray]
    a: int
    b: int
    cond: Optional[Tuple[int, int, int]]


class Program:
    """A compiled program (compiler::Compiled, src/compiler.rs:80-94)."""

    def __init__(self, handle: C.c_void_p, cregs):
        self._h = handle
        self.cregs = list(cregs)
        L = load()
        info = ProgramInfo()
        _check(L.zc_program_get_info(handle, C.byref(info)))
        self.n_qubits = info.n_qubits
        self.dynamic = bool(info.dynamic)
        self.stats = dict(input_gates=info.input_gates, cancelled=info.cancelled, output_ops=info.output_ops,
                          max_fused=info.max_fused)
        self.final_measures = []
        q, c = C.c_uint32(), C.c_uint32()
        for i in range(info.nfinal):
            _check(L.zc_program_get_final(handle, i, C.byref(q), C.byref(c)))
            self.final_measures.append((q.value, c.value))
        self._nops = info.nops

    @property
    def ops(self) -> List[Op]:
        L = load()
        out = []
        v = OpView()
        for i in range(self._nops):
            _check(L.zc_program_get_op(self._h, i, C.byref(v)))
            data = None
            if v.kind in (OP_UNITARY, OP_DIAG):
                n = (1 << (2 * v.k)) if v.kind == OP_UNITARY else (1 << v.k)
                data = np.ctypeslib.as_array(v.data, shape=(2 * n,)).view(np.complex128).copy()
            out.append(Op(v.kind, tuple(v.qubits[j] for j in range(v.k)), data, v.a, v.b,
                          (v.creg_offset, v.creg_len, v.value) if v.has_if else None))
        return out

    def __del__(self):
        try:
            if self._h:
                load().zc_program_free(self._h)
                self._h = None
        except Exception:
            pass


def encode(p: _circ.Program):
    ins = (Instr * max(1, len(p.instrs)))()
    for i, x in enumerate(p.instrs):
        z = ins[i]
        z.kind, z.cond_creg, z.cond_value = x.kind, x.cond_creg, x.cond_value
        z.name = x.name.encode()[:7]
        z.nq = len(x.qubits) if x.kind == _circ.I_GATE else 1
        z.np = len(x.params)
        for j, q in enumerate(x.qubits[:3]):
            z.q[j] = q
        for j, v in enumerate(x.params[:3]):
            z.p[j] = v
        z.clbit = x.clbit
    return ins, _u32([s for _, s in p.cregs])


def compile(p, fusion_max: int = 1, diag_max: int = 10, swap_perm: bool = True) -> Program:
    """compiler::compile (src/compiler.rs:118-200) with GB300 extensions."""
    if isinstance(p, _circ.Circuit):
        p = p.to_program()
    ins, cregs = encode(p)
    h = C.c_void_p()
    opts = CompileOptions(fusion_max, diag_max, 1 if swap_perm else 0)
    _check(load().zc_compile(p.n_qubits, cregs, len(p.cregs), ins, len(p.instrs), C.byref(opts), C.byref(h)))
    return Program(h, p.cregs)


@dataclass
class RunResult:
    """RunResult (src/exec.rs:115-130)."""

    counts: Dict[str, int]
    raw: Dict[int, int]
    shots: int
    n_qubits: int
    precision: int
    backend: str
    seed: int
    sim_time: float
    statevector: Optional[np.ndarray]
    stats: Dict[str, int]
    launches: int
    sweeps: int
    bytes_moved: int
    batched: bool = False
    notices: List[str] = field(default_factory=list)


def run(p, shots: int = 1024, seed: int = 0, precision: int = 0, fusion: Optional[int] = None,
        noise: Optional[NoiseModel] = None, statevector: bool = False, flags: int = FLAG_EXACT,
        program: Optional[Program] = None, sweep_high: int = 0) -> RunResult:
    """zeno::run_program with `--backend cuda` (src/lib.rs:224-250).

    Noisy runs compile with fusion 0 (src/lib.rs:228-231); the default dense
    fusion width on the GPU is 1 (diagonal fusion on)."""
    if isinstance(p, _circ.Circuit):
        p = p.to_program()
    noisy = noise is not None and not noise.is_trivial()
    if noisy:
        noise.validate()
    if program is None:
        program = compile(p, 0 if noisy else (1 if fusion is None else fusion))
    nz = NoiseC(*[getattr(noise, f.name) for f in fields(noise)]) if noisy else None
    opts = RunOptions(precision, flags, shots, seed, C.pointer(nz) if nz is not None else None, 0.0, sweep_high, 0)
    cap = max(16, min(shots, 1 << 22) + 1)
    keys = np.zeros(cap, dtype=np.uint64)
    counts = np.zeros(cap, dtype=np.uint64)
    sv = np.zeros(1 << p.n_qubits, dtype=np.complex128) if statevector else None
    res = RunResultC()
    _check(load().zc_run(program._h, C.byref(opts), C.byref(res), keys.ctypes.data_as(C.POINTER(C.c_uint64)),
                         counts.ctypes.data_as(C.POINTER(C.c_uint64)), cap,
                         sv.ctypes.data_as(C.POINTER(C.c_double)) if sv is not None else None))
    raw = {int(keys[i]): int(counts[i]) for i in range(min(res.n_keys, cap))}
    fmt: Dict[str, int] = {}
    for k, v in raw.items():
        key = _circ.format_key(k, p.cregs)
        fmt[key] = fmt.get(key, 0) + v
    prec = res.precision_bits
    return RunResult(fmt, raw, shots, p.n_qubits, prec, "cuda-f%d" % prec, seed, res.sim_seconds, sv,
                     program.stats, res.launches, res.sweeps, res.bytes_moved, bool(res.batched),
                     [x for x in res.notices.decode(errors="replace").split("\n") if x])


def device_info() -> Dict[str, object]:
    d = DeviceC()
    _check(load().zc_device_info(C.byref(d)))
    return {"name": d.name.decode(), "sms": d.sms, "compute_capability": "%d.%d" % (d.cc_major, d.cc_minor),
            "hbm_bytes": d.hbm_bytes, "free_bytes": d.free_bytes, "l2_bytes": d.l2_bytes}


def arith_peaks() -> Dict[str, float]:
    """FP64 / FP32 FMA issue rates of the current device (operations per
    second over the whole GPU), timed on issue-bound FMA loops."""
    d = ArithPeaksC()
    _check(load().zc_measure_arith_peaks(C.byref(d)))
    return {"fp64_fma_per_s": d.fp64_fma_per_s, "fp32_fma_per_s": d.fp32_fma_per_s, "sms": d.sms}


def device_budget(fraction: float = 0.75) -> int:
    """mem::budget_bytes (src/mem.rs:104-111): `fraction` of device_memory()."""
    out = C.c_uint64()
    _check(load().zc_device_budget(fraction, C.byref(out)))
    return out.value


def device_memory() -> int:
    """mem::physical_ram_bytes for the device: ZENO_MEM_BYTES, else total HBM."""
    out = C.c_uint64()
    _check(load().zc_device_memory(C.byref(out)))
    return out.value


def state_bytes(n: int, precision: int) -> int:
    return int(load().zc_state_bytes(n, precision))


def max_qubits(budget: int, precision: int) -> int:
    return int(load().zc_max_qubits(budget, precision))
