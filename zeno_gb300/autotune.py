"""Autotuner for the fusion width and the sweep tile shape.

zeno picks its dense fusion width from a fixed default (src/lib.rs:224-240,
fusion 3 on the CPU). On a GB300 the best width depends on the state's
precision and arithmetic mode: f64 gates are bound by the FP32 pipe in
double-float arithmetic, f32 sweeps by HBM or by instruction issue, and
fused k >= 4 blocks can go to the tensor cores. The tile shape of a sweep
(how many qubits above the 256-byte row a tile holds) trades ops per HBM
pass against the number of tiles in flight. Neither changes a result
beyond the arithmetic mode's own tolerance: exact mode is bit-identical at
every setting, because fusion is applied by the same compiler and sweeps
only group ops.

`tune(circuit, precision, flags)` times whole runs (no sampling) on the GPU
for each candidate (K, max_high) and returns the fastest; decisions are
cached per (qubits, precision, flags, circuit signature), in memory and, if
a path is given, in a JSON file. `run(...)` runs a circuit with the tuned
setting.
"""

import hashlib
import json
import os
import time
from typing import Callable, Dict, Iterable, List, Optional, Tuple

from . import backend as zb
from . import circuit as circ

_cache: Dict[str, Dict] = {}


def signature(p) -> str:
    """Stable digest of a program's instruction list (gate names, qubits, angles)."""
    h = hashlib.sha1()
    h.update(("%d|" % p.n_qubits).encode())
    for ins in p.instrs:
        h.update(repr((ins.kind, ins.name, tuple(ins.qubits), tuple(round(x, 12) for x in ins.params), ins.clbit,
                       ins.cond_creg, ins.cond_value)).encode())
    return h.hexdigest()[:16]


def key(n: int, precision: int, flags: int, sig: str) -> str:
    return "%d/%d/%d/%s" % (n, precision, flags, sig)


def candidates(n: int, precision: int, flags: int, fusions: Optional[Iterable[int]] = None,
               highs: Optional[Iterable[int]] = None) -> List[Tuple[int, int]]:
    """(K, max_high) pairs worth timing. K >= 4 only with tensor cores (f32),
    where fused blocks are GEMMs; without them dense blocks cost arithmetic
    the sweeps avoid. max_high 0 = the automatic shape."""
    if fusions is None:
        fusions = [1, 2, 3] + ([5, 6, 7] if precision == 32 and (flags & zb.FLAG_TENSOR) else [])
    if highs is None:
        highs = [0, 4, 5, 6, 7] if n >= 14 else [0]
    return [(k, h) for k in fusions for h in highs]


def search(cands: List[Tuple[int, int]], measure: Callable[[int, int], float], reps: int = 1,
           budget_s: Optional[float] = None) -> Tuple[Tuple[int, int], List[Dict]]:
    """Time every candidate (best of `reps`), stop early when the budget is
    spent; return the fastest and the table."""
    table = []
    t0 = time.perf_counter()
    for k, h in cands:
        best = min(measure(k, h) for _ in range(max(1, reps)))
        table.append({"fusion": k, "max_high": h, "seconds": best})
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
    win = min(table, key=lambda r: r["seconds"])
    return (win["fusion"], win["max_high"]), table


def tune(c, precision: int = 64, flags: int = zb.FLAG_FAST, fusions=None, highs=None, reps: int = 1,
         budget_s: Optional[float] = None, cache_path: Optional[str] = None) -> Dict:
    """Pick (fusion width, tile shape) for circuit `c` on this GPU."""
    p = c.to_program() if isinstance(c, circ.Circuit) else c
    k = key(p.n_qubits, precision, flags, signature(p))
    if cache_path and not _cache and os.path.exists(cache_path):
        with open(cache_path) as f:
            _cache.update(json.load(f))
    if k in _cache:
        return _cache[k]
    progs: Dict[int, zb.Program] = {}

    def measure(fusion: int, high: int) -> float:
        if fusion not in progs:
            progs[fusion] = zb.compile(p, fusion)
        r = zb.run(p, shots=0, seed=1, precision=precision, flags=flags, program=progs[fusion], sweep_high=high)
        return r.sim_time

    measure(*candidates(p.n_qubits, precision, flags, fusions, highs)[0])  # warm-up (allocator, module load)
    (fusion, high), table = search(candidates(p.n_qubits, precision, flags, fusions, highs), measure, reps, budget_s)
    out = {"fusion": fusion, "max_high": high, "table": table}
    _cache[k] = out
    if cache_path:
        with open(cache_path, "w") as f:
            json.dump(_cache, f, indent=1)
    return out


def run(c, shots: int = 1024, seed: int = 0, precision: int = 64, flags: int = zb.FLAG_FAST, **kw) -> zb.RunResult:
    """Run `c` with the tuned fusion width and tile shape."""
    t = tune(c, precision, flags, **kw)
    p = c.to_program() if isinstance(c, circ.Circuit) else c
    return zb.run(p, shots=shots, seed=seed, precision=precision, flags=flags, fusion=t["fusion"],
                  sweep_high=t["max_high"])
