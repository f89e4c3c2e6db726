"""Roofline denominators of the current GPU, measured.

  python -m zeno_gb300.peaks        # prints one JSON object

* HBM copy bandwidth: `MEASURED_PEAKS.json` at the repository root
  (measured on the GB300s with a STREAM-style copy), else the
  6,800 GB/s fallback;
* FP64 and FP32 FMA issue rates: `zc_measure_arith_peaks` (issue-bound FMA
  loops in the library): double-float sweeps are bound by the FP32 pipe,
  exact f64 kernels by the FP64 pipe;
* TF32 tensor throughput: the best of a few cuBLAS TF32 GEMMs
  (8192 x 8192 x 8192 f32 with TF32 math), a plain library GEMM as the
  denominator of the 3xTF32 block path (three TF32 MMAs per algorithmic
  product, so its bound is this rate / 3).
"""

from __future__ import annotations

import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HBM_FALLBACK_GBS = 6800.0


def hbm_gbs():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def tf32_tflops(n: int = 8192, reps: int = 5) -> float:
    import torch

    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        c = torch.empty(n, n, device="cuda", dtype=torch.float32)
        torch.matmul(a, b, out=c)
        best = 0.0
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            e1.synchronize()
            best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        del a, b, c
        torch.cuda.empty_cache()
        return best
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def measure(with_tf32: bool = True):
    from . import backend as zb

    zb.load()
    hbm, src = hbm_gbs()
    ar = zb.arith_peaks()
    out = {"hbm_gbs": hbm, "hbm_source": src, "fp64_fma_per_s": ar["fp64_fma_per_s"],
           "fp32_fma_per_s": ar["fp32_fma_per_s"], "sms": ar["sms"]}
    if with_tf32:
        out["tf32_tflops"] = tf32_tflops()
    return out


if __name__ == "__main__":
    print(json.dumps(measure()))
