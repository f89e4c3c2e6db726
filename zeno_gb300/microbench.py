"""Kernel micro-benchmarks for the GB300 backend (CUDA-event timing).

  python -m zeno_gb300.microbench [--qubits 28 30] [--fp-peaks]
  python -m zeno_gb300.microbench --sweep-costs 26

Per state size, precision and arithmetic mode: one-qubit gate passes on
low and high qubits, CX, a 3-qubit diagonal, dense k-qubit blocks, a sweep
of 1/4/7 one-qubit gates, sampling and prob_one; each reported as time and
algorithmic GB/s (2S per pass, S for CX). `--fp-peaks` prints the FP64 /
FP32 FMA issue rates and the TF32 GEMM rate (zeno_gb300/peaks.py). `--sweep-costs N`
prints the cost of one micro-op of each kind inside a sweep.
"""

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def fp_peaks():
    from . import peaks

    print(json.dumps(peaks.measure()))


def timed(be, torch, fn, reps=3):
    s = torch.cuda.ExternalStream(be.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    be.finish()
    e0.record(s)
    for _ in range(reps):
        fn()
    be.finish()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def timed_flush(be, torch, fn, reps=3):
    """Device time per call of fn followed by a flush (one sweep per call)."""
    s = torch.cuda.ExternalStream(be.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    be.finish()
    e0.record(s)
    for _ in range(reps):
        fn()
        be.finish()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def kernels(qubits):
    import torch

    from . import backend as zc

    zc.load()
    rng = np.random.default_rng(0)

    def unitary(d):
        return np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0]

    for n in qubits:
        for prec in (64, 32):
            for flags, mode in ((zc.FLAG_EXACT, "exact"), (zc.FLAG_FAST, "fast")):
                be = zc.CudaBackend(n, prec, flags | zc.FLAG_NO_SWEEPS)
                S = (1 << n) * prec // 8 * 2
                row = lambda name, ms, b: print("n=%d f%d %-5s %-14s %9.3f ms %7.0f GB/s" % (n, prec, mode, name, ms,
                                                                                         b / ms / 1e6), flush=True)
                for q in (0, 3, n - 1):
                    u = unitary(2)
                    row("1q q=%d" % q, timed(be, torch, lambda: be.apply_unitary([q], u)), 2 * S)
                row("cx", timed(be, torch, lambda: be.apply_cx(3, n - 2)), S)
                d = np.exp(1j * np.arange(8))
                row("diag3", timed(be, torch, lambda: be.apply_diagonal([2, 7, n - 1], d)), 2 * S)
                for k in (2, 4):
                    u = unitary(1 << k)
                    qs = list(range(1, 2 * k, 2))
                    row("kq%d" % k, timed(be, torch, lambda: be.apply_unitary(qs, u), 2), 2 * S)
                row("sample 1024", timed(be, torch, lambda: be.sample(1024, 1), 2), S)
                row("prob_one", timed(be, torch, lambda: be.prob_one(n - 1), 2), S / 2)
                be.close()
                be = zc.CudaBackend(n, prec, flags)
                for g in (1, 4, 7):
                    us = [unitary(2) for _ in range(g)]
                    ms = timed(be, torch, lambda: [be.apply_unitary([q], us[i]) for i, q in enumerate(range(n - g, n))])
                    row("sweep of %d 1q" % g, ms, 2 * S)
                be.close()


def sweep_costs(n):
    """Cost of one micro-op of each kind inside a sweep: a flush of 1 and of
    32 ops of that kind (one sweep each, same tile), per-op time = the
    difference / 31, per amplitude in ns and in SM cycles at 2.07 GHz."""
    import torch

    from . import backend as zc

    zc.load()
    rng = np.random.default_rng(1)

    def unitary(d):
        return np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))[0]

    kinds = {
        "u1 q=1 (row bit)": lambda be, i: be.apply_unitary([1], unitary(2)),
        "u1 q=n-1 (high bit)": lambda be, i: be.apply_unitary([n - 1], unitary(2)),
        "u1 alternating q=0,n-1,n-2": lambda be, i: be.apply_unitary([(0, n - 1, n - 2)[i % 3]], unitary(2)),
        "cx 2->n-1": lambda be, i: be.apply_cx(2, n - 1),
        "swap 1<->n-2": lambda be, i: be.apply_swap(1, n - 2),
        "diag1 q=n-1": lambda be, i: be.apply_diagonal([n - 1], np.exp(1j * rng.uniform(0, 6.3, 2))),
        "diag4": lambda be, i: be.apply_diagonal([0, 3, n - 2, n - 1], np.exp(1j * rng.uniform(0, 6.3, 16))),
        "diag10": lambda be, i: be.apply_diagonal(list(range(0, 20, 2)), np.exp(1j * rng.uniform(0, 6.3, 1024))),
    }
    for prec, flags, mode in ((32, zc.FLAG_FAST, "fma"), (32, zc.FLAG_EXACT, "exact"), (64, zc.FLAG_FAST, "df"),
                              (64, zc.FLAG_EXACT, "exact")):
        be = zc.CudaBackend(n, prec, flags)
        for name, f in kinds.items():
            t1 = timed_flush(be, torch, lambda: f(be, 0))
            t32 = timed_flush(be, torch, lambda: [f(be, i) for i in range(32)])
            per = (t32 - t1) / 31
            ns_amp = per * 1e6 / (1 << n)
            print("n=%d f%d %-5s %-28s sweep(1) %8.3f ms  sweep(32) %8.3f ms  per op %7.3f ms  %6.3f ns/amp  "
                  "%6.1f SM-cycles/amp/SM" % (n, prec, mode, name, t1, t32, per, ns_amp, ns_amp * 2.07 * 152),
                  flush=True)
        be.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--qubits", type=int, nargs="*", default=[28, 30])
    ap.add_argument("--fp-peaks", action="store_true")
    ap.add_argument("--sweep-costs", type=int, default=0, metavar="N", help="per-micro-op costs at N qubits")
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(HERE))
    if a.fp_peaks:
        fp_peaks()
    if a.sweep_costs:
        sweep_costs(a.sweep_costs)
    elif a.qubits:
        kernels(a.qubits)


if __name__ == "__main__":
    main()
