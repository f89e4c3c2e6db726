"""Continuous-batching serving on one GB300 (include/zeno_cuda_serve.h).

`Server` wraps the C engine: submit compiled programs, `step()` admits
requests by HBM footprint, advances every admitted request in one packed
launch and completes the finished ones. `serve_stream` drives it with a
timed arrival stream and reports circuits/s and p50/p99 latency;
`plain_stream` runs the same stream one circuit per call (zeno's model:
one `run_program` at a time, FIFO) for comparison. `request_stream` builds
the synthetic workload: Poisson arrivals, qubits log-uniform over 8..26,
gate-mix circuits of depth U[4, 60], shots log-uniform over 1..8192, f64
escalation for a flagged fraction, all seeds from a master seed.
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import backend as zb
from . import circuit as circ
from .rng import Xoshiro256pp, splitmix64


# Entry points of include/zeno_cuda_serve.h.
EXPORTS = ("zc_server_create", "zc_server_destroy", "zc_server_submit", "zc_server_step", "zc_server_done_ids",
           "zc_server_take")


class ServerOptions(C.Structure):
    _fields_ = [("pool_bytes", C.c_uint64), ("max_slots", C.c_uint32), ("flags", C.c_uint32)]


class ServerStatus(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("pending", "active", "done", "launches", "packed_launches", "admitted",
                                          "completed", "pool_used", "steps", "plan_us", "sample_us",
                                          "wait_us", "device_us")]


_bound = False


def _lib():
    global _bound
    L = zb.load()
    if not _bound:
        vp, u32, u64, i32, P = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.POINTER
        L.zc_server_create.argtypes = [P(ServerOptions), P(vp)]
        L.zc_server_create.restype = i32
        L.zc_server_destroy.argtypes = [vp]
        L.zc_server_destroy.restype = None
        L.zc_server_submit.argtypes = [vp, vp, i32, u64, u64, P(u64)]
        L.zc_server_submit.restype = i32
        L.zc_server_step.argtypes = [vp, P(ServerStatus)]
        L.zc_server_step.restype = i32
        L.zc_server_done_ids.argtypes = [vp, P(u64), C.c_size_t, P(C.c_size_t)]
        L.zc_server_done_ids.restype = i32
        L.zc_server_take.argtypes = [vp, u64, P(u64), u64, P(u64)]
        L.zc_server_take.restype = i32
        _bound = True
    return L


class Server:
    def __init__(self, pool_bytes: int = 0, max_slots: int = 0, flags: int = zb.FLAG_FAST):
        L = _lib()
        h = C.c_void_p()
        zb._check(L.zc_server_create(C.byref(ServerOptions(pool_bytes, max_slots, flags)), C.byref(h)))
        self._h = h
        self.status = ServerStatus()

    def submit(self, program: "zb.Program", precision: int, shots: int, seed: int) -> int:
        rid = C.c_uint64()
        zb._check(_lib().zc_server_submit(self._h, program._h, precision, shots, seed, C.byref(rid)))
        return rid.value

    def step(self) -> ServerStatus:
        zb._check(_lib().zc_server_step(self._h, C.byref(self.status)))
        return self.status

    def done_ids(self) -> List[int]:
        n = C.c_size_t()
        zb._check(_lib().zc_server_done_ids(self._h, None, 0, C.byref(n)))
        arr = (C.c_uint64 * max(1, n.value))()
        zb._check(_lib().zc_server_done_ids(self._h, arr, n.value, C.byref(n)))
        return [arr[i] for i in range(n.value)]

    def take(self, rid: int, shots: int) -> np.ndarray:
        out = np.zeros(max(1, shots), dtype=np.uint64)
        n = C.c_uint64()
        zb._check(_lib().zc_server_take(self._h, rid, out.ctypes.data_as(C.POINTER(C.c_uint64)), shots,
                                        C.byref(n)))
        return out[: n.value]

    def close(self):
        if getattr(self, "_h", None):
            _lib().zc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def counts_from_indices(idx: np.ndarray, program: "zb.Program") -> Dict[str, int]:
    """run_sampled's histogram (src/exec.rs:437-449) from sampled indices."""
    raw: Dict[int, int] = {}
    for b, c in zip(*np.unique(idx, return_counts=True)):
        cl = 0
        for q, cb in program.final_measures:
            cl = (cl & ~(1 << cb)) | (((int(b) >> q) & 1) << cb)
        raw[cl] = raw.get(cl, 0) + int(c)
    out: Dict[str, int] = {}
    for k, v in raw.items():
        key = circ.format_key(k, program.cregs)
        out[key] = out.get(key, 0) + v
    return out


@dataclass
class Request:
    arrival: float
    n: int
    depth: int
    shots: int
    seed: int
    precision: int
    program: object = None
    rid: int = 0
    done: float = 0.0
    counts: Optional[Dict[str, int]] = None


def request_stream(count: int, rate: float, master_seed: int = 2024, f64_fraction: float = 0.05,
                   n_min: int = 8, n_max: int = 26) -> List[Request]:
    """Poisson arrivals at `rate` req/s; n = floor(n_min * ((n_max+1)/n_min)^u),
    depth = range(4, 61), shots = floor(exp(u * ln 8192)), f64 if u < f64_fraction;
    request i draws from xoshiro256++ seeded with splitmix64(master_seed + i)."""
    g = Xoshiro256pp(master_seed)
    t = 0.0
    out = []
    for i in range(count):
        t += -math.log(1.0 - g.f64()) / rate
        r = Xoshiro256pp(splitmix64(master_seed + i))
        n = min(n_max, int(n_min * ((n_max + 1) / n_min) ** r.f64()))
        depth = r.range(4, 61)
        shots = max(1, min(8192, int(math.exp(r.f64() * math.log(8192)))))
        prec = 64 if r.f64() < f64_fraction else 32
        out.append(Request(t, n, depth, shots, r.next_u64(), prec))
    return out


def compile_requests(reqs: List[Request]) -> None:
    for q in reqs:
        q.program = zb.compile(circ.mixed_circuit(q.n, q.depth, q.seed).to_program(), 1)


def serve_stream(reqs: List[Request], flags: int = zb.FLAG_FAST, pool_bytes: int = 0, max_slots: int = 0,
                 keep_counts: bool = False) -> Dict[str, float]:
    """Replay the arrival stream against the server in real time."""
    srv = Server(pool_bytes, max_slots, flags)
    by_id = {}
    pending = sorted(reqs, key=lambda q: q.arrival)
    i = 0
    t0 = time.perf_counter()
    done = 0
    step_s = 0.0
    while done < len(reqs):
        now = time.perf_counter() - t0
        while i < len(pending) and pending[i].arrival <= now:
            q = pending[i]
            q.rid = srv.submit(q.program, q.precision, q.shots, q.seed)
            by_id[q.rid] = q
            i += 1
        ts = time.perf_counter()
        st = srv.step()
        step_s += time.perf_counter() - ts
        for rid in srv.done_ids():
            q = by_id[rid]
            idx = srv.take(rid, q.shots)
            q.done = time.perf_counter() - t0
            if keep_counts:
                q.counts = counts_from_indices(idx, q.program)
            done += 1
        if st.active == 0 and st.pending == 0 and i < len(pending):
            wait = pending[i].arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.01))
    wall = time.perf_counter() - t0
    stats = _latency_stats(reqs, wall)
    stats["launches"] = srv.status.launches
    stats["packed_launches"] = srv.status.packed_launches
    stats["steps"] = srv.status.steps
    stats["host_s"] = {"plan_launch": srv.status.plan_us * 1e-6, "sample": srv.status.sample_us * 1e-6,
                       "wait_device": srv.status.wait_us * 1e-6, "in_step": step_s}
    stats["device_busy_s"] = srv.status.device_us * 1e-6
    srv.close()
    return stats


def plain_stream(reqs: List[Request], flags: int = zb.FLAG_FAST, keep_counts: bool = False) -> Dict[str, float]:
    """One circuit per call, FIFO in arrival order (each request runs alone)."""
    t0 = time.perf_counter()
    moved, sweeps, sim = 0, 0, 0.0
    for q in sorted(reqs, key=lambda q: q.arrival):
        now = time.perf_counter() - t0
        if q.arrival > now:
            time.sleep(q.arrival - now)
        shell = circ.Program(q.n, list(q.program.cregs), [])  # registers only: the program is compiled
        r = zb.run(shell, shots=q.shots, seed=q.seed, precision=q.precision, flags=flags, program=q.program)
        q.done = time.perf_counter() - t0
        moved += r.bytes_moved
        sweeps += r.sweeps
        sim += r.sim_time
        if keep_counts:
            q.counts = r.counts
    wall = time.perf_counter() - t0
    stats = _latency_stats(reqs, wall)
    # state traffic of the sweeps and per-op passes (the packed server moves the same bytes)
    stats.update(bytes_moved=moved, sweeps=sweeps, sim_seconds=sim)
    return stats


def _latency_stats(reqs: List[Request], wall: float) -> Dict[str, float]:
    lat = np.array([q.done - q.arrival for q in reqs])
    return {"requests": len(reqs), "wall_s": wall, "circuits_per_s": len(reqs) / wall,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}
