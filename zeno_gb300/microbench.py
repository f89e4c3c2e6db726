"""Kernel micro-benchmarks for the GB300 backend (CUDA-event timing).

  python -m zeno_gb300.microbench [--qubits 28 30] [--fp-peaks]

Per state size, precision and arithmetic mode: one-qubit gate passes on
low and high qubits, CX, a 3-qubit diagonal, dense k-qubit blocks, a sweep
of 1/4/7 one-qubit gates, sampling and prob_one; each reported as time and
algorithmic GB/s (2S per pass, S for CX). `--fp-peaks` compiles and runs
probes/fp_peaks.cu (FP64 and FP32 instruction rates).
"""

import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def fp_peaks():
    from .build import ARCH, nvcc

    src = os.path.join(HERE, "probes", "fp_peaks.cu")
    exe = os.path.join(HERE, "_lib", "fp_peaks")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    subprocess.run([nvcc()] + ARCH + ["-O3", "-o", exe, src], check=True)
    print(subprocess.run([exe], check=True, capture_output=True, text=True).stdout, end="")


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--qubits", type=int, nargs="*", default=[28, 30])
    ap.add_argument("--fp-peaks", action="store_true")
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(HERE))
    if a.fp_peaks:
        fp_peaks()
    if a.qubits:
        kernels(a.qubits)


if __name__ == "__main__":
    main()
