"""Benchmark: 30-qubit depth-40 f64 circuit on one GB300 (zeno's state-vector hot path).

Workload: u3(theta, phi, lambda) with U[0, 2pi) angles on every qubit, then CX
on a seeded random perfect matching, 40 layers, 30 qubits, f64 split-complex
state (16 GiB, far larger than L2, so no flush is needed between steps),
measure all, 1024 shots. One step = one circuit: reset to |0...0>, every
compiled op, then sampling.

Prints ONE JSON line (rank 0). `value` = circuits/s with the op stream
resident on the device side of the API; `e2e` = the same through
`zc_run` (state allocation, op tables host->device, kernels, sampling,
indices device->host). `roofline` = the dominant kernel's algorithmic HBM
bytes per launch over its CUDA-event duration; `cpu_baseline` = the oracle
(the C restatement of zeno's CPU backend) on all host cores for a bounded
sample of the same workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
# DRAM read+write per launch over algorithmic bytes, from an ncu capture of
# the f64 double-float sweep kernel at 26 qubits (state 8x the L2):
# 1.074 GB read + 1.027 GB write against 2S = 2.147 GB.
MEASURED_TRAFFIC_RATIO = {"sweep": (1.074e9 + 1.027e9) / 2.147e9}
# The same capture: issue slots 58% busy, FMA pipe 37%, ALU pipe 31%, FP64 0%.
SWEEP_DF_PIPES = {"issue_active_pct": 57.6, "fma_pipe_pct": 36.5, "alu_pipe_pct": 30.9, "fp64_pipe_pct": 0.0}
# FP32 instructions per amplitude of each double-float sweep micro-op
# (zeno_gb300/csrc/zc_arith.cuh): a product is 4 (FMUL + 3 FFMA), TwoSum 6,
# renormalisation 3. Complex 2x2: four 4-term dot products per pair
# (4*4 + 3*6 + 6 + 3 = 43 each) = 86; real 2x2 and one-qubit diagonals:
# 2-term dot products (2*4 + 6 + 2 + 3 = 19), two per amplitude = 38. Register
# passes chain unnormalised pairs: table diagonal 2 x (2*4 + 6 + 2) = 32,
# rotation [[1, -t], [t, 1]] 2 x (4 + 6 + 2) = 24 (one renormalisation per
# sweep, where the tile goes back to f64, is not counted). CX and SWAP move
# data only.
DF_FP32_INSTR_PER_AMP = {"complex": 86, "diag1": 38, "diag_table": 32, "cx": 0, "swap": 0, "real": 38,
                         "rotation": 24}
FP32_INSTR_PEAK = 34.3e12  # measured FMA issue rate (zeno_gb300/probes/fp_peaks.cu)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=40)
    ap.add_argument("--precision", type=int, default=64)
    ap.add_argument("--fusion", type=int, default=1)
    ap.add_argument("--mode", default="fast", choices=["exact", "fast"])
    ap.add_argument("--shots", type=int, default=1024)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--cpu-layers", type=int, default=1, help="layers timed for the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-check", action="store_true", help="skip the fast-vs-exact accuracy check")
    ap.add_argument("--check-qubits", type=int, default=26)
    ap.add_argument("--no-extras", action="store_true", help="skip the batched-trajectory measurement")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def workload_name(a):
    arith = {"exact": "exact (reference expression trees, native FP)",
             "fast": "fast (double-float on the FP32 pipe, f64 storage)" if a.precision == 64 else "fast (FMA)"}
    return "%dq depth-%d u3+matching-CX f%d, %d shots, fusion %d, %s arithmetic" % (
        a.qubits, a.depth, a.precision, a.shots, a.fusion, arith[a.mode])


def accuracy_check(a, zc, C):
    """Fast mode against exact mode (bit-identical to the FP64 oracle) on the
    same circuit family at `check_qubits`: max |d amp| and output TVD."""
    import numpy as np

    p = C.matching_circuit(a.check_qubits, a.depth, a.seed).to_program()
    ex = zc.run(p, shots=0, precision=a.precision, statevector=True, flags=zc.FLAG_EXACT).statevector
    fa = zc.run(p, shots=0, precision=a.precision, statevector=True, flags=zc.FLAG_FAST).statevector
    d = float(np.abs(ex - fa).max())
    tvd = float(0.5 * np.abs(np.abs(ex) ** 2 - np.abs(fa) ** 2).sum())
    return {"qubits": a.check_qubits, "depth": a.depth, "max_abs_damp": d, "tvd": tvd,
            "reference": "exact mode (bit-identical to the FP64 oracle in the parity tests)",
            "tolerance": {"max_abs_damp": 1e-12 if a.precision == 64 else 1e-5, "tvd": 1e-6}}


def batched_trajectories(zc, C):
    """16 qubits, depth 20, depolarizing 1e-3 (1q) / 1e-2 (CX), damping 1e-3,
    2% readout, 4096 trajectories in one launch vs the per-shot replay."""
    noise = zc.NoiseModel(depolarizing_1q=1e-3, depolarizing_2q=1e-2, amplitude_damping=1e-3,
                          readout_flip_0to1=0.02, readout_flip_1to0=0.02)
    p = C.matching_circuit(16, 20, 7).to_program()
    prog = zc.compile(p, 0)
    zc.run(p, shots=256, seed=1, precision=32, noise=noise, program=prog)
    t0 = time.perf_counter()
    r = zc.run(p, shots=4096, seed=2, precision=32, noise=noise, program=prog)
    tb = time.perf_counter() - t0
    plain_shots = 32
    t0 = time.perf_counter()
    zc.run(p, shots=plain_shots, seed=2, precision=32, noise=noise, program=prog, flags=zc.FLAG_PER_SHOT)
    tp = (time.perf_counter() - t0) / plain_shots
    return {"workload": "16q depth-20 u3+matching-CX f32, dep 1e-3/1e-2, damping 1e-3, readout 2%, 4096 trajectories",
            "trajectories_per_s": 4096 / tb, "seconds": tb, "launches": r.launches, "batched": r.batched,
            "plain_per_shot_trajectories_per_s": 1.0 / tp, "plain_sample_shots": plain_shots,
            "speedup_vs_plain": (4096 / tb) * tp}


def serving_sample(zc):
    """A short request stream (8..22 qubits, gate-mix circuits, Poisson
    arrivals at 3000 req/s): the continuous-batching server against one
    circuit per call in arrival order."""
    from zeno_gb300 import serve

    reqs = serve.request_stream(300, rate=3000.0, master_seed=2024, n_max=22)
    serve.compile_requests(reqs)
    s = serve.serve_stream(reqs)
    plain = serve.request_stream(300, rate=3000.0, master_seed=2024, n_max=22)
    for a, b in zip(plain, reqs):
        a.program = b.program
    pl = serve.plain_stream(plain)
    return {"workload": "300 requests, 8..22 qubits, depth U[4,60], shots 1..8192, Poisson 3000 req/s, 5% f64",
            "server": s, "one_per_call": pl, "throughput_ratio": s["circuits_per_s"] / pl["circuits_per_s"]}


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(a, threads=None):
    """The oracle on the host cores for a bounded sample: state allocation,
    `cpu_layers` layers of the circuit and the sampler, scaled to one circuit."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    from zeno_gb300 import circuit as C

    oracle.build()
    oracle.set_threads(threads or os.cpu_count() or 1)
    nthreads = oracle.threads()
    layer = C.matching_circuit(a.qubits, a.cpu_layers, a.seed, measure=False).to_program()
    comp = oracle.compile(layer, a.fusion)
    t0 = time.perf_counter()
    st = oracle.State(a.qubits, a.precision)
    t1 = time.perf_counter()
    for op in comp.ops:
        st.apply_op(op)
    t2 = time.perf_counter()
    st.sample(a.shots, 1)
    t3 = time.perf_counter()
    st.close()
    per_circuit = (t1 - t0) + (t2 - t1) * a.depth / a.cpu_layers + (t3 - t2)
    return {
        "value": 1.0 / per_circuit, "unit": "circuits/s", "cores": nthreads, "kind": "port",
        "sample": "%d of %d layers (%d ops) + state allocation + %d-shot sampling on %d threads, "
                  "layer time scaled x%d" % (a.cpu_layers, a.depth, len(comp.ops), a.shots, nthreads,
                                              a.depth // a.cpu_layers),
        "seconds_sampled": t3 - t0,
    }


def dist_init(a):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch.distributed as dist

    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    import torch

    if torch.cuda.is_available():
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        dist.init_process_group("gloo")
    return rank, ws, local


def job_throughput(units_per_rank, seconds, ws):
    """Whole-job rate of `ws` replicas: every rank did `units_per_rank` units;
    the job took the slowest rank's time (max over ranks)."""
    if ws > 1:
        import torch
        import torch.distributed as dist

        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(seconds)], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        seconds = float(t.item())
    return units_per_rank * ws / seconds, seconds


def reference_arm(a):
    rank, ws, _ = dist_init(a)
    if rank != 0:
        return
    steps = []
    for i in range(a.warmup + a.steps):
        r = cpu_baseline(a)
        if i >= a.warmup:
            steps.append(r)
    v = statistics.median(s["value"] for s in steps)
    line = {
        "impl": "reference", "metric": "30q circuit throughput (u3 + matching-CX, depth 40, f64)",
        "value": v, "unit": "circuits/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if a.precision == 64 else "f32", "data": "synthetic (seeded circuit)",
        "config": {"workload": workload_name(a), "l2": "state 16 GiB > L2, no flush needed"},
        "cpu_baseline": {k: steps[-1][k] for k in ("kind", "cores", "sample")} | {"value": v,
                                                                                 "unit": "circuits/s"},
        "e2e": {"value": v, "unit": "circuits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "C restatement of zeno's scalar CPU backend (the Rust binary cannot be built here)",
    }
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        return reference_arm(a)
    rank, ws, local = dist_init(a)
    import torch

    from zeno_gb300 import backend as zc
    from zeno_gb300 import build as zb
    from zeno_gb300 import circuit as C
    from zeno_gb300.rng import splitmix64

    if rank == 0:
        zb.build()
    if ws > 1:
        torch.distributed.barrier()
    zc.load()
    dev = local
    torch.cuda.set_device(dev)
    flags = zc.FLAG_FAST if a.mode == "fast" else zc.FLAG_EXACT
    circ = C.matching_circuit(a.qubits, a.depth, a.seed).to_program()
    prog = zc.compile(circ, a.fusion)
    ops = prog.ops
    be = zc.CudaBackend(a.qubits, a.precision, flags)
    stream = torch.cuda.ExternalStream(be.stream())
    S = (1 << a.qubits) * (a.precision // 8) * 2
    sample_seed = splitmix64(a.seed)

    def step():
        be.reset_all()
        for op in ops:
            if op.kind == zc.OP_UNITARY:
                be.apply_unitary(op.qubits, op.data)
            elif op.kind == zc.OP_DIAG:
                be.apply_diagonal(op.qubits, op.data)
            elif op.kind == zc.OP_CX:
                be.apply_cx(op.a, op.b)
            elif op.kind == zc.OP_SWAP:
                be.apply_swap(op.a, op.b)
        return be.sample(a.shots, sample_seed)

    for _ in range(a.warmup):
        step()
    be.finish()
    c0 = be.counters()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    be.profile(True)  # CUDA events around every launch, on the backend's stream
    with Clocks(dev) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for k in range(a.steps):
            step()
        t_end.record(stream)
        be.finish()
        torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    elapsed = t_start.elapsed_time(t_end) / 1000.0
    c1 = be.counters()
    classes = be.profile_read()
    be.profile(False)
    value, elapsed = job_throughput(a.steps, elapsed, ws)
    gates_ms = sum(d["ms"] for d in classes.values())  # all of our kernels in the timed region
    mops = {k: c1["micro_ops"][k] - c0["micro_ops"][k] for k in c1["micro_ops"]}
    fp32_instr = sum(n * DF_FP32_INSTR_PER_AMP[k] for k, n in mops.items()) * float(1 << a.qubits)
    dom = max(classes, key=lambda c: classes[c]["ms"])
    dd = classes[dom]
    peak, peak_kind = peaks()
    achieved = (dd["bytes"] / dd["launches"]) / (dd["ms"] / dd["launches"] / 1000.0) / 1e9
    line = {
        "metric": "30q circuit throughput (u3 + matching-CX, depth 40, f64)",
        "value": value, "unit": "circuits/s", "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": elapsed / a.steps * 1000.0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if a.precision == 64 else "f32",
        "data": "synthetic (seeded circuit, random angles)",
        "config": {"workload": workload_name(a), "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "state %.0f GiB > 129 MB L2: no flush needed" % (S / 2**30),
                   "ops": len(ops), "input_gates": prog.stats["input_gates"]},
        "gpu_launches": int(c1["launches"] - c0["launches"]),
        "gpu_busy_frac": gates_ms / 1000.0 / elapsed,
        "amp_updates_per_s": {"value": prog.stats["input_gates"] * 2.0 ** a.qubits * value,
                              "definition": "input gates x 2^n per second, the throughput zeno bench prints "
                                            "(src/main.rs:1138)"},
        "kernels": {c: {"launches": d["launches"], "avg_ms": d["ms"] / d["launches"],
                        "GBps": (d["bytes"] / d["launches"]) / (d["ms"] / d["launches"] / 1000.0) / 1e9
                        if d["bytes"] else None,
                        "share": d["ms"] / gates_ms} for c, d in sorted(classes.items())},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "bytes_per_launch": dd["bytes"] / dd["launches"],
                     "traffic": (MEASURED_TRAFFIC_RATIO[dom] * dd["bytes"] / dd["launches"]
                                 if dom in MEASURED_TRAFFIC_RATIO else None),
                     "ops_per_launch": len(ops) * a.steps / dd["launches"] if dom == "sweep" else 1.0,
                     "limiter": ("FP32/ALU issue: each sweep applies many gates per HBM pass in double-float "
                                 "arithmetic; ncu at 26q: %s" % SWEEP_DF_PIPES)
                     if dom == "sweep" and a.mode == "fast" and a.precision == 64 else None,
                     "compute": ({"bound": "fp32_pipe", "unit": "FP32 instr/s",
                                  "achieved": fp32_instr / (dd["ms"] / 1e3),
                                  "peak": FP32_INSTR_PEAK,
                                  "frac": fp32_instr / (dd["ms"] / 1e3) / FP32_INSTR_PEAK,
                                  "micro_ops": mops,
                                  "count": "sweep micro-ops issued in the timed steps x FP32 instructions per "
                                           "amplitude of their double-float arithmetic %s; index arithmetic, "
                                           "data moves and f64 <-> double-float conversions not counted"
                                           % DF_FP32_INSTR_PER_AMP})
                     if dom == "sweep" and a.mode == "fast" and a.precision == 64 else None},
        "clocks": clk.summary(),
    }
    if not a.no_e2e:
        torch.cuda.synchronize()
        be.close()
        h2d = 0
        for op in ops:
            if op.kind in (zc.OP_UNITARY, zc.OP_DIAG):
                h2d += op.data.size * 2 * (a.precision // 8)
        h2d += a.shots * 8
        d2h = a.shots * 8 + max(1, (1 << a.qubits) >> 16) * 8
        zc.run(circ, shots=a.shots, seed=a.seed, precision=a.precision, flags=flags, program=prog)
        ts = []
        for _ in range(max(1, min(a.steps, 2))):
            t0 = time.perf_counter()
            r = zc.run(circ, shots=a.shots, seed=a.seed, precision=a.precision, flags=flags, program=prog)
            ts.append(time.perf_counter() - t0)
        e2e_value, _ = job_throughput(1, statistics.median(ts), ws)
        line["e2e"] = {"value": e2e_value, "unit": "circuits/s", "h2d_bytes_per_step": h2d,
                       "d2h_bytes_per_step": d2h, "sim_seconds": r.sim_time,
                       "path": "zc_run: allocate state, per-op host->device tables, kernels, sample, read indices"}
    if rank == 0 and not a.no_extras:
        line["batched_trajectories"] = batched_trajectories(zc, C)
        line["serving"] = serving_sample(zc)
    if rank == 0 and a.mode == "fast" and not a.no_check:
        line["accuracy"] = accuracy_check(a, zc, C)
    if rank == 0 and not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline(a)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
