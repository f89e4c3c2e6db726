"""Measurement suite for the workloads beside the headline benchmark.

  python -m zeno_gb300.suite qft        # QFT 24/28 qubits, f64/f32, exact/fast, 8192 shots
  python -m zeno_gb300.suite fusion     # 30q depth-40 f64 at fusion widths K = 1..5
  python -m zeno_gb300.suite big        # 33q depth-40 f64 (128 GiB state)
  python -m zeno_gb300.suite serving    # request stream at several arrival rates, server vs one-per-call
  python -m zeno_gb300.suite trajectories  # 4096 noisy 16q trajectories, batched vs per-shot
  python -m zeno_gb300.suite tc         # 28q gate mix fused to k=5..7 blocks on tensor cores vs FP64
  python -m zeno_gb300.suite gatemix    # 28q gate mix on plain sweeps, f32 and f64 fast (device time)
  python -m zeno_gb300.suite sampler    # sample / prob_one per state size, exact and fast
  python -m zeno_gb300.suite tune       # autotuner tables (fusion width x tile shape), 26 qubits
  python -m zeno_gb300.suite dynamic    # 16q dynamic circuit, 4096 shots: batched trajectories vs per-shot

Each prints JSON lines. Times are wall-clock around complete runs
(`zc_run`: state allocation, ops, sampling), the semantics of zeno's
sim_time (src/exec.rs:372-381).
"""

import argparse
import json
import math
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from zeno_gb300 import backend as zb  # noqa: E402
from zeno_gb300 import circuit as C  # noqa: E402


def _run(p, prog, prec, flags, shots, seed):
    t0 = time.perf_counter()
    r = zb.run(p, shots=shots, seed=seed, precision=prec, flags=flags, program=prog)
    return time.perf_counter() - t0, r


def qft(args):
    for n in ((args.qubits,) if args.qubits else (24, 28)):
        c, x = C.qft_circuit(n, 11)
        p = c.to_program()
        prog = zb.compile(p, 1)
        for prec in args.precisions:
            for flags, mode in ((zb.FLAG_EXACT, "exact"), (zb.FLAG_FAST, "fast")):
                if mode not in args.modes:
                    continue
                _run(p, prog, prec, flags, 8192, 3)
                t, r = _run(p, prog, prec, flags, 8192, 3)
                print(json.dumps({"workload": "qft", "qubits": n, "precision": prec, "mode": mode, "seconds": t,
                                  "sweeps": r.sweeps, "launches": r.launches, "ops": len(prog.ops),
                                  "input_gates": r.stats["input_gates"],
                                  "amp_updates_per_s": r.stats["input_gates"] * 2.0 ** n / t}), flush=True)


def fusion(args):
    n = args.qubits
    p = C.matching_circuit(n, 40, 7).to_program()
    for k in args.fusions:
        prog = zb.compile(p, k)
        for flags, mode in ((zb.FLAG_FAST, "fast"),):
            t, r = _run(p, prog, 64, flags, 1024, 7)
            S = 2.0 ** n * 16
            print(json.dumps({"workload": "%dq d40 f64" % n, "fusion": k, "mode": mode, "seconds": t,
                              "ops": len(prog.ops), "max_fused": prog.stats["max_fused"], "sweeps": r.sweeps,
                              "launches": r.launches, "sweep_GBps": r.bytes_moved / t / 1e9,
                              "state_GiB": S / 2**30}), flush=True)


def big(args):
    n = args.qubits
    p = C.matching_circuit(n, 40, 7).to_program()
    prog = zb.compile(p, 1)
    t, r = _run(p, prog, 64, zb.FLAG_FAST, 1024, 7)
    print(json.dumps({"workload": "%dq d40 f64 fast" % n, "seconds": t, "sweeps": r.sweeps,
                      "launches": r.launches, "state_GiB": 2.0 ** n * 16 / 2**30,
                      "hbm_GBps_of_passes": r.bytes_moved / t / 1e9}), flush=True)


def serving(args):
    from zeno_gb300 import serve

    for rate in args.rates:
        reqs = serve.request_stream(args.requests, rate=rate, master_seed=2024, n_max=args.n_max)
        serve.compile_requests(reqs)
        s = serve.serve_stream(reqs)
        if args.server_only:
            print(json.dumps({"workload": "serving", "rate_per_s": rate, "requests": args.requests,
                              "qubits": [8, args.n_max], "server": s}), flush=True)
            continue
        reqs2 = serve.request_stream(args.requests, rate=rate, master_seed=2024, n_max=args.n_max)
        for a, b in zip(reqs2, reqs):
            b_prog = b.program
            a.program = b_prog
        pl = serve.plain_stream(reqs2)
        print(json.dumps({"workload": "serving", "rate_per_s": rate, "requests": args.requests,
                          "qubits": [8, args.n_max], "server": s, "plain": pl,
                          "throughput_ratio": s["circuits_per_s"] / pl["circuits_per_s"]}), flush=True)


def trajectories(args):
    noise = zb.NoiseModel(depolarizing_1q=1e-3, depolarizing_2q=1e-2, amplitude_damping=1e-3,
                          readout_flip_0to1=0.02, readout_flip_1to0=0.02)
    p = C.matching_circuit(16, 20, 7).to_program()
    prog = zb.compile(p, 0)
    zb.run(p, shots=256, seed=1, precision=32, noise=noise, program=prog)
    t0 = time.perf_counter()
    r = zb.run(p, shots=4096, seed=2, precision=32, noise=noise, program=prog)
    tb = time.perf_counter() - t0
    t0 = time.perf_counter()
    zb.run(p, shots=32, seed=2, precision=32, noise=noise, program=prog, flags=zb.FLAG_PER_SHOT)
    tp = (time.perf_counter() - t0) / 32
    print(json.dumps({"workload": "16q d20 noisy, 4096 trajectories", "batched_seconds": tb,
                      "trajectories_per_s": 4096 / tb, "per_shot_trajectories_per_s": 1 / tp,
                      "launches": r.launches, "keys": len(r.counts)}), flush=True)


def _apply_ops(be, prog):
    for op in prog.ops:
        if op.kind == zb.OP_UNITARY:
            be.apply_unitary(list(op.qubits), op.data.reshape(1 << len(op.qubits), -1))
        elif op.kind == zb.OP_DIAG:
            be.apply_diagonal(list(op.qubits), op.data)
        elif op.kind == zb.OP_CX:
            be.apply_cx(op.a, op.b)
        else:
            be.apply_swap(op.a, op.b)


def tc(args):
    """28q depth-60 gate mix fused to 5/6/7-qubit blocks on tensor cores (f32,
    3xTF32) against the FP64 plain run on the GPU: accuracy from full runs,
    device time per kernel class from the in-library profiler."""
    import numpy as np

    n = args.qubits
    p = C.mixed_circuit(n, 60, 7).to_program()
    ref_prog = zb.compile(p, 1)
    ref = zb.run(p, shots=0, seed=1, precision=64, flags=zb.FLAG_FAST, statevector=True, program=ref_prog)
    S = 2.0 ** n * 8  # f32 state bytes
    for k in (5, 6, 7):
        prog = zb.compile(p, k)
        r = zb.run(p, shots=0, seed=1, precision=32, flags=zb.FLAG_TENSOR | zb.FLAG_FAST, statevector=True,
                   program=prog)
        d = float(np.abs(r.statevector - ref.statevector).max())
        tvd = float(0.5 * np.abs(np.abs(r.statevector) ** 2 - np.abs(ref.statevector) ** 2).sum())
        be = zb.CudaBackend(n, 32, zb.FLAG_TENSOR | zb.FLAG_FAST)
        _apply_ops(be, prog)
        be.finish()
        be.profile(True)
        _apply_ops(be, prog)
        be.finish()
        prof = be.profile_read()
        be.close()
        blocks = [op for op in prog.ops if op.kind == zb.OP_UNITARY and len(op.qubits) >= 4]
        flops = sum(8.0 * 2.0 ** (n + len(op.qubits)) for op in blocks)
        kq = prof.get("tc_block", {"launches": 0, "ms": 0.0})
        dev_ms = sum(v["ms"] for v in prof.values())
        print(json.dumps({"workload": "%dq d60 gate mix, fused k=%d, f32 3xTF32" % (n, k),
                          "device_ms": dev_ms, "tc_blocks": kq["launches"], "tc_ms": kq["ms"],
                          "tc_ms_per_block": kq["ms"] / max(1, kq["launches"]),
                          "tc_TFLOPs_algorithmic": flops / (kq["ms"] * 1e-3) / 1e12 if kq["ms"] else None,
                          "tc_GBps": 2 * S * kq["launches"] / (kq["ms"] * 1e-3) / 1e9 if kq["ms"] else None,
                          "kernels_ms": {k2: round(v["ms"], 3) for k2, v in prof.items()},
                          "ops": len(prog.ops), "max_abs_damp_vs_f64": d, "tvd_vs_f64": tvd}), flush=True)
    prog1 = zb.compile(p, 1)
    be = zb.CudaBackend(n, 32, zb.FLAG_FAST)
    _apply_ops(be, prog1)
    be.finish()
    be.profile(True)
    _apply_ops(be, prog1)
    be.finish()
    prof = be.profile_read()
    be.close()
    r = zb.run(p, shots=0, seed=1, precision=32, flags=zb.FLAG_FAST, statevector=True, program=prog1)
    d = float(np.abs(r.statevector - ref.statevector).max())
    print(json.dumps({"workload": "%dq d60 gate mix, unfused sweeps f32 FMA" % n,
                      "device_ms": sum(v["ms"] for v in prof.values()),
                      "kernels_ms": {k2: round(v["ms"], 3) for k2, v in prof.items()},
                      "ops": len(prog1.ops), "max_abs_damp_vs_f64": d}), flush=True)


def gatemix(args):
    """The depth-60 gate mix on plain sweeps (fusion 1), f32 and f64 fast:
    device time per kernel class from the in-library profiler."""
    from . import workloads as W

    n = args.qubits
    p = C.mixed_circuit(n, 60, 7).to_program()
    prog = zb.compile(p, 1)
    for prec in (32, 64):
        d = W.device_profile(n, prec, zb.FLAG_FAST, prog, 1, 1, 6800.0)
        print(json.dumps({"workload": "%dq d60 gate mix, f%d fast sweeps" % (n, prec), "ops": len(prog.ops),
                          "device_ms": d["device_ms"], "kernels": d["kernels"]}), flush=True)


def sampler(args):
    """Sampler and reductions per state size, exact and fast mode: wall time of
    one 1024-shot sample and one prob_one, and the per-kernel device times
    (in-library CUDA-event profiler) of two samples, one prob_one, one norm."""
    import numpy as np

    h = np.array([[1, 1], [1, -1]], dtype=complex) / np.sqrt(2)
    for prec in (64, 32):
        for flags, mode in ((zb.FLAG_EXACT, "exact"), (zb.FLAG_FAST, "fast")):
            for n in args.sizes:
                be = zb.CudaBackend(n, prec, flags)
                for q in range(n):
                    be.apply_unitary([q], h)
                be.norm_sqr()
                be.profile(True)
                for _ in range(2):
                    be.sample(1024, 5)
                be.prob_one(n - 1)
                be.norm_sqr()
                prof = be.profile_read()
                be.profile(False)
                t0 = time.perf_counter()
                be.sample(1024, 5)
                ts = time.perf_counter() - t0
                t0 = time.perf_counter()
                be.prob_one(n - 1)
                tp = time.perf_counter() - t0
                print(json.dumps({"workload": "sampler", "qubits": n, "precision": prec, "mode": mode,
                                  "sample_1024_ms": ts * 1e3, "prob_one_ms": tp * 1e3,
                                  "kernels_ms": {k: [v["launches"], round(v["ms"], 3)] for k, v in prof.items()}}),
                      flush=True)
                be.close()


def dynamic(args):
    """Dynamic circuit (mid-circuit measure + conditional gate + reset after
    every layer): all shots as batched trajectories vs zeno's per-shot replay."""
    import math

    import numpy as np

    n, layers, shots = args.qubits, 6, 4096
    rng = np.random.default_rng(21)
    cregs = [("m%d" % i, 1) for i in range(layers)] + [("f", n)]
    p = C.Program(n, cregs, [])
    for layer in range(layers):
        for q in range(n):
            p.instrs.append(C.Instr(C.I_GATE, "u3", (q,), tuple(float(x) for x in rng.uniform(0, 2 * math.pi, 3))))
        for q in range(layer % 2, n - 1, 2):
            p.instrs.append(C.Instr(C.I_GATE, "cx", (q, q + 1)))
        mq = int(rng.integers(n))
        p.instrs.append(C.Instr(C.I_MEASURE, qubits=(mq,), clbit=layer))
        p.instrs.append(C.Instr(C.I_GATE, "x", ((mq + 1) % n,), (), 0, layer, 1))
        p.instrs.append(C.Instr(C.I_RESET, qubits=(mq,)))
    for q in range(n):
        p.instrs.append(C.Instr(C.I_MEASURE, qubits=(q,), clbit=layers + q))
    prog = zb.compile(p, 0)
    zb.run(p, shots=64, seed=1, precision=32, program=prog)
    t0 = time.perf_counter()
    r = zb.run(p, shots=shots, seed=2, precision=32, program=prog)
    tb = time.perf_counter() - t0
    per = 32
    t0 = time.perf_counter()
    zb.run(p, shots=per, seed=2, precision=32, program=prog, flags=zb.FLAG_PER_SHOT)
    tp = (time.perf_counter() - t0) / per
    print(json.dumps({"workload": "%dq %d-layer dynamic circuit (measure + if + reset per layer), %d shots"
                      % (n, layers, shots), "batched": r.batched, "batched_seconds": tb,
                      "shots_per_s": shots / tb, "per_shot_shots_per_s": 1 / tp, "speedup": tp * shots / tb,
                      "launches": r.launches, "keys": len(r.counts)}), flush=True)


def tune(args):
    """Autotuner tables: fusion width x tile shape, timed whole runs."""
    from . import autotune as at

    n = args.qubits
    cases = [("%dq d40 u3+matching-CX f64 fast" % n, C.matching_circuit(n, 40, 7), 64, zb.FLAG_FAST),
             ("%dq d40 u3+matching-CX f32 fast" % n, C.matching_circuit(n, 40, 7), 32, zb.FLAG_FAST),
             ("%dq d60 gate mix f32 fast + tensor cores" % n, C.mixed_circuit(n, 60, 7), 32,
              zb.FLAG_FAST | zb.FLAG_TENSOR)]
    for name, c, prec, flags in cases:
        t = at.tune(c, prec, flags)
        print(json.dumps({"workload": name, "best_fusion": t["fusion"], "best_max_high": t["max_high"],
                          "table": t["table"]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["qft", "fusion", "big", "serving", "trajectories", "tc", "gatemix", "sampler",
                                       "tune", "dynamic"])
    ap.add_argument("--sizes", type=int, nargs="*", default=[16, 20, 22, 26, 28, 30])
    ap.add_argument("--qubits", type=int, default=None)
    ap.add_argument("--requests", type=int, default=1000)
    ap.add_argument("--rates", type=float, nargs="*", default=[100.0, 1000.0, 10000.0])
    ap.add_argument("--n-max", type=int, default=26)
    ap.add_argument("--server-only", action="store_true", help="serving: skip the one-circuit-per-call arm")
    ap.add_argument("--fusions", type=int, nargs="*", default=[1, 2, 3, 4, 5], help="fusion: widths K to run")
    ap.add_argument("--precisions", type=int, nargs="*", default=[64, 32], help="qft: state precisions to run")
    ap.add_argument("--modes", nargs="*", default=["exact", "fast"], choices=["exact", "fast"],
                    help="qft: arithmetic modes to run")
    a = ap.parse_args()
    if a.qubits is None:
        a.qubits = {"fusion": 30, "big": 33, "tc": 28, "gatemix": 28, "tune": 26, "dynamic": 16}.get(a.what, 30)
    zb.load()
    globals()[a.what](a)


if __name__ == "__main__":
    main()
