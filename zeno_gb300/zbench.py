"""`zeno bench --backend cuda` (src/main.rs:1105-1230) on the GPU.

  python -m zeno_gb300.zbench [--qubits 20,22,24,26] [--depth 12] [--fusion K]
                              [--precision auto|f32|f64] [--arith exact|fast]
                              [--seed 7] [--compare-fusion] [--json]

Sweeps zeno's own `random_circuit` (u3 on every qubit, then an alternating
CX ladder; src/circuit.rs:152-174) over qubit counts, one shot each, and
reports what zeno's bench reports — input gates, output ops, sim time,
amp-updates/s (input gates x 2^n / sim time, src/main.rs:1138), the
no-fusion speed-up with --compare-fusion — in zeno's schema-v1 JSON
(src/main.rs:1167-1230, keys kept as they are). Each result adds the GPU's
own figures: state passes, kernel launches, the algorithmic HBM bytes of
those passes per second (`pass_GBps`: 2S per pass, S for a standalone CX or
SWAP) and its fraction of the measured HBM copy peak. Sizes whose state
exceeds the device budget are skipped with zeno's reason text
(src/main.rs:1113-1118), as ZENO_MEM_BYTES lets a test pretend.
"""

from __future__ import annotations

import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from zeno_gb300 import backend as zb  # noqa: E402
from zeno_gb300 import circuit as C  # noqa: E402
from zeno_gb300.info import FRACTION, human  # noqa: E402
from zeno_gb300.peaks import hbm_gbs  # noqa: E402


def parse(argv=None):
    ap = argparse.ArgumentParser(prog="zeno bench --backend cuda")
    ap.add_argument("--qubits", default="20,22,24,26", help="qubit counts to sweep, comma-separated")
    ap.add_argument("--depth", type=int, default=12)
    ap.add_argument("--fusion", type=int, default=None, help="dense fused-gate width 0-7 [default: 1]")
    ap.add_argument("--precision", default="auto", choices=["auto", "f32", "f64"])
    ap.add_argument("--arith", default="exact", choices=["exact", "fast"])
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--compare-fusion", action="store_true")
    ap.add_argument("--json", action="store_true")
    a = ap.parse_args(argv)
    a.qubit_list = [int(x) for x in a.qubits.split(",") if x.strip()]
    return a


def _chip():
    try:
        return zb.device_info()["name"]
    except zb.ZenoCudaError:
        return "unknown"


def bench(a) -> dict:
    budget = zb.device_budget(FRACTION)
    # auto precision falls back to f32, so a size only exceeds the budget when
    # even f32 does (src/main.rs:1107-1112)
    check_prec = 64 if a.precision == "f64" else 32
    prec = {"auto": 0, "f32": 32, "f64": 64}[a.precision]
    flags = zb.FLAG_FAST if a.arith == "fast" else zb.FLAG_EXACT
    fusion = 1 if a.fusion is None else a.fusion
    peak, peak_src = hbm_gbs()
    results, notes = [], []
    for n in a.qubit_list:
        needed = zb.state_bytes(n, check_prec) if n <= 48 else float("inf")
        if n > 48 or needed > budget:
            results.append({"qubits": n, "skipped": True,
                            "reason": "needs %s, budget %s" % (human(needed) if n <= 48 else "more than 2^48 amplitudes",
                                                                human(budget))})
            continue
        p = C.random_circuit(n, a.depth, a.seed).to_program()
        prog = zb.compile(p, fusion)
        r = zb.run(p, shots=1, seed=a.seed, precision=prec, flags=flags, program=prog)
        for note in r.notices:
            if not note.startswith("circuit has no measurements") and note not in notes:
                notes.append(note)
        secs = max(r.sim_time, 1e-9)
        gbs = r.bytes_moved / secs / 1e9
        row = {"qubits": n, "skipped": False, "input_gates": prog.stats["input_gates"],
               "output_ops": prog.stats["output_ops"], "sim_time_ms": secs * 1e3,
               "amp_updates_per_s": prog.stats["input_gates"] * 2.0 ** n / secs,
               "precision": "f%d" % r.precision, "backend": r.backend,
               "passes": r.sweeps, "launches": r.launches, "pass_GBps": gbs, "hbm_roofline_frac": gbs / peak}
        if a.compare_fusion:
            r0 = zb.run(p, shots=1, seed=a.seed, precision=prec, flags=flags, program=zb.compile(p, 0))
            row["nofusion_time_ms"] = r0.sim_time * 1e3
            row["speedup"] = max(r0.sim_time, 1e-9) / secs
        results.append(row)
    return {"schema_version": 1, "chip": _chip(), "threads": os.cpu_count() or 1, "depth": a.depth,
            "fusion": fusion, "fusion_auto": a.fusion is None, "seed": a.seed, "precision": a.precision,
            "backend": "cuda", "arith": a.arith, "hbm_peak_GBps": peak, "hbm_peak_source": peak_src,
            "results": results, "notices": notes}


def main(argv=None):
    a = parse(argv)
    out = bench(a)
    if a.json:
        print(json.dumps(out, indent=2))
        return
    print("zeno bench · %s · cuda · %s arithmetic · depth %d · fusion %s%d" % (
        out["chip"], a.arith, a.depth, "auto " if a.fusion is None else "", out["fusion"]))
    print("%7s %8s %6s %12s %16s %10s %8s" % ("qubits", "gates", "ops", "time", "amp-updates/s", "GB/s", "of HBM"))
    for r in out["results"]:
        if r["skipped"]:
            print("%7d  skipped: %s" % (r["qubits"], r["reason"]))
            continue
        print("%7d %8d %6d %9.2f ms %16.3e %10.1f %7.1f%%" % (
            r["qubits"], r["input_gates"], r["output_ops"], r["sim_time_ms"], r["amp_updates_per_s"],
            r["pass_GBps"], 100 * r["hbm_roofline_frac"]))
    for n in out["notices"]:
        print("note: " + n)


if __name__ == "__main__":
    main()
