"""Benchmark: 30-qubit depth-40 f64 circuit on one GB300 (zeno's state-vector hot path).

Workload: u3(theta, phi, lambda) with U[0, 2pi) angles on every qubit, then CX
on a seeded random perfect matching, 40 layers, 30 qubits, f64 split-complex
state (16 GiB, far larger than L2, so no flush is needed between steps),
measure all, 1024 shots, fusion 1. One step = one circuit: reset to
|0...0>, every compiled op, then sampling.

Prints ONE JSON line (rank 0). `value` = circuits/s with the op stream
resident on the device side of the API, fast arithmetic (double-float on
the FP32 pipe, f64 storage; within 1e-12 of the FP64 oracle); `e2e` = the
same through `zc_run` (state allocation, op tables host->device, kernels,
sampling, indices device->host); `exact_mode` = the same circuit in the
drop-in's default exact arithmetic (bit-identical to zeno's CPU kernels).
`roofline` = the dominant kernel's algorithmic HBM bytes per launch over its
CUDA-event duration; `cpu_baseline` = the oracle (the C restatement of
zeno's CPU backend) on all host cores for a bounded sample of the same
workload. `configs` = every other seeded workload at its own shape
(zeno_gb300/workloads.py).

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

METRIC = "30q circuit throughput (u3 + matching-CX, depth 40, f64)"
# DRAM read+write per launch over algorithmic bytes, from an ncu capture of
# the f64 double-float sweep kernel at 26 qubits (state 8x the L2; the sweeps
# between the first and the last of a flush, which hand the state over as
# packed double-float pairs): 1.074 GB read + 1.029 GB write against
# 2S = 2.147 GB.
MEASURED_TRAFFIC_RATIO = {"sweep": (1.074e9 + 1.029e9) / 2.147e9}
# The same capture: issue slots 50-51% busy, FMA pipe 30-31% of its
# instruction peak and 46% of its cycles (packed f32x2 rotations), ALU pipe
# 24-25%, FP64 0%.
SWEEP_DF_PIPES = {"issue_active_pct": 49.6, "fma_pipe_pct": 30.0, "fma_pipe_cycles_pct": 46.2, "alu_pipe_pct": 24.3,
                  "fp64_pipe_pct": 0.0}
# FP32 operations per amplitude of each double-float sweep micro-op
# (zeno_gb300/csrc/zc_arith.cuh; rotations issue them as packed f32x2
# instructions, two operations each): a product is 4 (MUL + 3 FMA), TwoSum 6,
# renormalisation 3. Complex 2x2: four 4-term dot products per pair
# (4*4 + 3*6 + 6 + 3 = 43 each) = 86; real 2x2 and one-qubit diagonals:
# 2-term dot products (2*4 + 6 + 2 + 3 = 19), two per amplitude = 38. Register
# passes chain unnormalised pairs: table diagonal 2 x (2*4 + 6 + 2) = 32,
# rotation [[1, -t], [t, 1]] 2 x (4 + 6 + 2) = 24 (one renormalisation per
# sweep, where the tile goes back to f64, is not counted). CX and SWAP move
# data only.
DF_FP32_OPS_PER_AMP = {"complex": 86, "diag1": 38, "diag_table": 32, "cx": 0, "swap": 0, "real": 38,
                         "rotation": 24}
CONFIG_NAMES = ("matching_20q", "qft", "fusion_sweep", "big_state", "trajectories", "gate_mix_tc", "serving")


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
    ap.add_argument("--validate-qubits", type=int, default=24,
                    help="reference arm: full circuit timed at this size against its per-layer projection")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-exact", action="store_true", help="skip the exact-mode circuit")
    ap.add_argument("--no-check", action="store_true", help="skip the fast-vs-exact accuracy check")
    ap.add_argument("--check-qubits", type=int, default=26)
    ap.add_argument("--configs", default="all",
                    help="comma list of %s, 'all' or 'none'" % ",".join(CONFIG_NAMES))
    return ap.parse_args()


def headline_config(a):
    """The workload, identical in both arms' lines (the arithmetic is reported
    beside it, under `arithmetic`)."""
    S = (1 << a.qubits) * (a.precision // 8) * 2
    return {"workload": "%dq depth-%d u3+matching-CX f%d, %d shots, fusion %d" % (
        a.qubits, a.depth, a.precision, a.shots, a.fusion),
        "l2": "state %.0f GiB > 129 MB L2: no flush needed" % (S / 2**30)}


def arithmetic_name(mode, precision):
    if mode == "exact":
        return "exact: zeno's expression trees, separately rounded, no FMA (bit-identical to its CPU kernels)"
    if precision == 64:
        return "fast: double-float (FP32 pairs) on the FP32 pipe, f64 storage; within 1e-12 of the FP64 oracle"
    return "fast: FMA-contracted f32; within 1e-5 of the FP64 oracle"


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


# ---------------------------------------------------------------- CPU legs
# (the oracle is loaded only here: the CPU baseline of our line and the
# reference arm)


def _oracle(threads=None):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.build()
    oracle.set_threads(threads or os.cpu_count() or 1)
    return oracle


def layer_programs(a, qubits):
    """The headline circuit cut into its `depth` layers (n u3 + n/2 CX each),
    each compiled with the oracle's compiler at the headline's fusion. For
    this circuit nothing fuses across a layer boundary (a CX on every qubit
    separates one layer's u3 from the next), so the layers' ops are the whole
    circuit's ops."""
    from zeno_gb300 import circuit as C

    oracle = _oracle()
    p = C.matching_circuit(qubits, a.depth, a.seed, measure=False).to_program()
    per = len(p.instrs) // a.depth
    out = []
    for layer in range(a.depth):
        lp = C.Program(qubits, [], p.instrs[layer * per:(layer + 1) * per])
        out.append(oracle.compile(lp, a.fusion))
    return out


def cpu_baseline(a, threads=None):
    """The oracle on the host cores for a bounded sample: state allocation,
    `cpu_layers` layers of the circuit and the sampler, scaled to one circuit."""
    from zeno_gb300 import circuit as C

    oracle = _oracle(threads)
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


def cpu_trajectories(shots=256):
    """The oracle's per-shot noisy path (zeno's run_per_shot, parallel over
    shots on every host core) on the trajectory workload: 16 qubits, depth
    20, f32, the same noise model; a bounded sample of `shots` trajectories."""
    from zeno_gb300 import circuit as C
    from zeno_gb300 import workloads as W

    oracle = _oracle()

    class _Noise:
        pass

    nz = _Noise()
    for f, _ in oracle.ZoNoise._fields_:
        setattr(nz, f, 0.0)
    for k, v in W.TRAJ_NOISE.items():
        setattr(nz, k, v)
    p = C.matching_circuit(16, 20, 7).to_program()
    t0 = time.perf_counter()
    oracle.run(p, prec=32, shots=shots, seed=2, noise=nz)
    t = time.perf_counter() - t0
    return {"value": shots / t, "unit": "trajectories/s", "cores": oracle.threads(), "kind": "port",
            "sample": "%d trajectories of the same workload (per-shot replay, parallel over shots)" % shots,
            "seconds_sampled": t}


def reference_arm(a):
    """zeno's CPU backend (the oracle port, all host threads) on the headline
    circuit. A step is one layer of the circuit applied to a persistent 30q
    state (40 consecutive steps are one whole circuit); state allocation, the
    first layer and the 1024-shot sampling are timed once. value = 1 circuit /
    (allocation + first layer + 39 x mean later layer + sampling).
    Validation: the whole 40-layer circuit timed at `validate_qubits` against
    the same projection."""
    rank, ws, _ = dist_init(a)
    if rank != 0:
        return
    oracle = _oracle()
    nthreads = oracle.threads()

    def project(qubits, steps, warmup):
        layers = layer_programs(a, qubits)
        t0 = time.perf_counter()
        st = oracle.State(qubits, a.precision)
        t_alloc = time.perf_counter() - t0
        ts_all = []
        for i in range(warmup + steps):
            c = layers[i % a.depth]
            t0 = time.perf_counter()
            for op in c.ops:
                st.apply_op(op)
            ts_all.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        st.sample(a.shots, 1)
        t_sample = time.perf_counter() - t0
        st.close()
        # the first layer also pays the first touch of the zeroed pages
        # (zeno's zero_state is a calloc too); it is timed, not projected
        ts = ts_all[max(1, warmup):]
        layer_s = statistics.mean(ts)
        circuit = t_alloc + ts_all[0] + (a.depth - 1) * layer_s + t_sample
        return t_alloc, ts_all[0], layer_s, t_sample, ts, layers, circuit

    # validation at a smaller size: full circuit vs projection
    _, _, _, _, _, layers_v, proj_v = project(a.validate_qubits, 3, 1)
    t0 = time.perf_counter()
    st = oracle.State(a.validate_qubits, a.precision)
    for c in layers_v:
        for op in c.ops:
            st.apply_op(op)
    st.sample(a.shots, 1)
    full_v = time.perf_counter() - t0
    st.close()

    t_alloc, first_s, layer_s, t_sample, ts, _, per_circuit = project(a.qubits, a.steps, a.warmup)
    v = 1.0 / per_circuit
    sample = ("one layer (%d u3 + %d CX) of the %d-layer circuit per step on a persistent %dq state, %d threads; "
              "allocation, the first layer (first touch of the zeroed state) and %d-shot sampling timed once; "
              "circuit = allocation + first layer + %d x mean later layer + sampling"
              % (a.qubits, a.qubits // 2, a.depth, a.qubits, nthreads, a.shots, a.depth - 1))
    line = {
        "impl": "reference", "metric": METRIC,
        "value": v, "unit": "circuits/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": statistics.mean(ts) * 1000.0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if a.precision == 64 else "f32",
        "data": "synthetic (seeded circuit, random angles)",
        "config": headline_config(a),
        "arithmetic": arithmetic_name("exact", a.precision),
        "cpu_baseline": {"kind": "port", "cores": nthreads, "sample": sample, "value": v, "unit": "circuits/s"},
        "e2e": {"value": v, "unit": "circuits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "step_unit": "one circuit layer (1/%d of a circuit)" % a.depth,
        "extrapolated": True,
        "measured": {"layers_timed": len(ts), "layer_seconds_mean": layer_s,
                     "layer_seconds_min": min(ts), "layer_seconds_max": max(ts),
                     "allocation_seconds": t_alloc, "first_layer_seconds": first_s,
                     "sampling_seconds": t_sample,
                     "circuit_seconds_projected": per_circuit},
        "validation": {"qubits": a.validate_qubits, "full_circuit_seconds": full_v,
                       "projected_seconds": proj_v, "projected_over_full": proj_v / full_v},
        "note": "C restatement of zeno's scalar CPU backend (the Rust binary cannot be built here)",
    }
    print(json.dumps(line), flush=True)


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


def run_configs(a, peak, pk, line):
    from zeno_gb300 import workloads as W

    want = CONFIG_NAMES if a.configs == "all" else () if a.configs == "none" else tuple(
        x for x in a.configs.split(",") if x)
    out = {}
    for name in want:
        t0 = time.perf_counter()
        try:
            if name == "gate_mix_tc":
                out[name] = W.gate_mix_tc(peak, pk.get("tf32_tflops"))
            else:
                out[name] = getattr(W, name)(peak)
        except Exception as e:  # one failing workload must not hide the others
            out[name] = {"error": "%s: %s" % (type(e).__name__, e)}
        if isinstance(out[name], dict):
            out[name]["bench_wall_s"] = time.perf_counter() - t0
        else:
            out[name] = {"rows": out[name], "bench_wall_s": time.perf_counter() - t0}
    if "trajectories" in out and not a.no_cpu:
        out["trajectories"]["cpu_baseline"] = cpu_trajectories()
        t = out["trajectories"]
        if "trajectories_per_s" in t:
            t["speedup_vs_cpu_baseline"] = t["trajectories_per_s"] / t["cpu_baseline"]["value"]
    line["configs"] = out


def main():
    a = parse()
    if a.impl == "reference":
        return reference_arm(a)
    rank, ws, local = dist_init(a)
    import torch

    from zeno_gb300 import backend as zc
    from zeno_gb300 import build as zb
    from zeno_gb300 import circuit as C
    from zeno_gb300 import peaks
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
    pk = peaks.measure(with_tf32=rank == 0 and a.configs != "none")
    peak, peak_kind = pk["hbm_gbs"], pk["hbm_source"]
    be = zc.CudaBackend(a.qubits, a.precision, flags)
    stream = torch.cuda.ExternalStream(be.stream())
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
    fp32_ops = sum(n * DF_FP32_OPS_PER_AMP[k] for k, n in mops.items()) * float(1 << a.qubits)
    dom = max(classes, key=lambda c: classes[c]["ms"])
    dd = classes[dom]
    achieved = (dd["bytes"] / dd["launches"]) / (dd["ms"] / dd["launches"] / 1000.0) / 1e9
    df_sweep = dom == "sweep" and a.mode == "fast" and a.precision == 64
    line = {
        "metric": METRIC,
        "value": value, "unit": "circuits/s", "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": elapsed / a.steps * 1000.0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if a.precision == 64 else "f32",
        "data": "synthetic (seeded circuit, random angles)",
        "config": headline_config(a),
        "arithmetic": arithmetic_name(a.mode, a.precision),
        "parallelism": "replicas" if ws > 1 else "single",
        "ops": len(ops), "input_gates": prog.stats["input_gates"],
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
                     "limiter": ("double-float arithmetic on the FP32 pipe, not HBM: each sweep applies many "
                                 "gates per HBM pass; the rest is barrier and L1 latency; ncu at 26q: %s"
                                 % SWEEP_DF_PIPES) if df_sweep else None,
                     "compute": ({"bound": "fp32_pipe", "unit": "FP32 op/s",
                                  "achieved": fp32_ops / (dd["ms"] / 1e3),
                                  "peak": pk["fp32_fma_per_s"], "peak_source": "measured live (zc_measure_arith_peaks)",
                                  "frac": fp32_ops / (dd["ms"] / 1e3) / pk["fp32_fma_per_s"],
                                  "micro_ops": mops,
                                  "count": "sweep micro-ops issued in the timed steps x FP32 operations per "
                                           "amplitude of their double-float arithmetic %s (a packed f32x2 "
                                           "instruction is two); index arithmetic, data moves and f64 <-> "
                                           "double-float conversions not counted" % DF_FP32_OPS_PER_AMP})
                     if df_sweep else None},
        "peaks": pk,
        "clocks": clk.summary(),
    }
    torch.cuda.synchronize()
    be.close()
    if not a.no_e2e:
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
    if rank == 0 and a.mode == "fast" and not a.no_exact:
        # the drop-in's default (zc_create): exact arithmetic, one whole circuit
        t0 = time.perf_counter()
        r = zc.run(circ, shots=a.shots, seed=a.seed, precision=a.precision, flags=zc.FLAG_EXACT, program=prog)
        t = time.perf_counter() - t0
        line["exact_mode"] = {"workload": headline_config(a)["workload"], "arithmetic": arithmetic_name("exact", 64),
                              "seconds": t, "circuits_per_s": 1.0 / t, "sim_seconds": r.sim_time,
                              "sweeps": r.sweeps, "launches": r.launches,
                              "pass_GBps": r.bytes_moved / t / 1e9, "roofline_frac": r.bytes_moved / t / 1e9 / peak,
                              "fp64_fma_per_s_peak": pk["fp64_fma_per_s"],
                              "path": "zc_run through the drop-in's default arithmetic (ZC_FLAG_EXACT)"}
    if rank == 0 and a.mode == "fast" and not a.no_check:
        line["accuracy"] = accuracy_check(a, zc, C)
    if rank == 0 and a.configs != "none":
        run_configs(a, peak, pk, line)
    if rank == 0 and not a.no_cpu:
        line["cpu_baseline"] = cpu_baseline(a)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
