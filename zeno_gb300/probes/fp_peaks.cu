// Arithmetic throughput probe: FP64 and FP32 FMA / MUL / ADD instruction
// rates over the whole GPU (eight independent chains per thread, grid of
// 8 CTAs x 512 threads per SM). Prints instructions per second.
#include <cstdio>
#include <cuda_runtime.h>
template <typename T, int OP>
__global__ void k(T *out, T a, T b, int iters) {
    T x0 = threadIdx.x * (T)1e-7, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
#define STEP(x) if (OP == 0) x = fma(x, a, b); else if (OP == 1) x = x * a; else x = x + b;
        STEP(x0) STEP(x1) STEP(x2) STEP(x3) STEP(x4) STEP(x5) STEP(x6) STEP(x7)
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
template <typename T, int OP>
double run(int sms) {
    T *out; int blocks = sms * 8, threads = 512, iters = 4096;
    cudaMalloc(&out, sizeof(T) * blocks * threads);
    k<T, OP><<<blocks, threads>>>(out, (T)0.9999999, (T)1e-9, 16);
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0);
    k<T, OP><<<blocks, threads>>>(out, (T)0.9999999, (T)1e-9, iters);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    cudaFree(out);
    return (double)blocks * threads * iters * 8 / (ms * 1e-3);  // instructions/s
}
int main() {
    int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    printf("sms %d\n", sms);
    printf("f64 fma  %.3f Tinst/s\n", run<double, 0>(sms) / 1e12);
    printf("f64 mul  %.3f Tinst/s\n", run<double, 1>(sms) / 1e12);
    printf("f64 add  %.3f Tinst/s\n", run<double, 2>(sms) / 1e12);
    printf("f32 fma  %.3f Tinst/s\n", run<float, 0>(sms) / 1e12);
    printf("f32 mul  %.3f Tinst/s\n", run<float, 1>(sms) / 1e12);
    return 0;
}
