// Arithmetic issue rates of the current device: the compute denominators
// of the backend's rooflines (the double-float sweeps run on the FP32
// pipe, exact f64 kernels on the FP64 pipe). Every thread runs eight
// independent FMA chains, so the loop is issue-bound, not latency-bound.
#include <cuda_runtime.h>

#include "zc_internal.h"

namespace zc {
namespace {

constexpr int kPeakThreads = 512;
constexpr int kPeakCtasPerSm = 8;

template <typename T>
__global__ void __launch_bounds__(kPeakThreads) k_fma_chains(T *__restrict__ out, T a, T b, int iters) {
    T x0 = threadIdx.x * (T)1e-7, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
      x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b);
        x1 = fma(x1, a, b);
        x2 = fma(x2, a, b);
        x3 = fma(x3, a, b);
        x4 = fma(x4, a, b);
        x5 = fma(x5, a, b);
        x6 = fma(x6, a, b);
        x7 = fma(x7, a, b);
    }
    // one store per thread keeps the chains live; the grid matches `out`
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// FMA operations per second (one per thread per instruction) of one timed
// launch after a short warm-up launch.
template <typename T>
int fma_rate(int sms, int iters, double *rate) {
    const int blocks = sms * kPeakCtasPerSm;
    T *out = nullptr;
    ZC_CUDA(cudaMalloc(&out, sizeof(T) * (size_t)blocks * kPeakThreads));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        k_fma_chains<T><<<blocks, kPeakThreads>>>(out, (T)0.9999999, (T)1e-9, 16);
        e = cudaEventRecord(e0);
    }
    if (e == cudaSuccess) {
        k_fma_chains<T><<<blocks, kPeakThreads>>>(out, (T)0.9999999, (T)1e-9, iters);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return cuda_fail(e, "arithmetic peak probe");
    *rate = (double)blocks * kPeakThreads * (double)iters * 8.0 / (ms * 1e-3);
    return ZC_OK;
}

}  // namespace
}  // namespace zc

extern "C" int zc_measure_arith_peaks(zc_arith_peaks *out) {
    if (!out) return zc::fail(ZC_ERR_INVALID, "null output");
    int dev = 0, sms = 0;
    ZC_CUDA(cudaGetDevice(&dev));
    ZC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // FP64 issues ~68x slower than FP32 on this part: fewer iterations keep
    // both launches in the tens of milliseconds
    int rc = zc::fma_rate<double>(sms, 2048, &out->fp64_fma_per_s);
    if (rc != ZC_OK) return rc;
    rc = zc::fma_rate<float>(sms, 65536, &out->fp32_fma_per_s);
    if (rc != ZC_OK) return rc;
    out->sms = (uint32_t)sms;
    out->_pad = 0;
    return ZC_OK;
}
