// Shot sampling that allocates nothing.
//
// zc_sample keeps its chunk masses and its draw/index work area in device
// buffers that it grows with cudaMalloc on first use and whenever a larger
// state or shot count arrives. Some callers cannot let a library allocate at
// that point: an embedding runtime that carves all device memory into its
// own pool at start-up and forbids later cudaMalloc, or a serving loop that
// must not stall on cudaMalloc / cudaFree (cudaFree synchronises the
// device). zc_sample_noalloc draws the indices zeno's own sampler draws —
// those of zc_sample on an exact-mode state, whatever arithmetic flag this
// state was created with — but all of its device scratch lives in one
// file-scope __device__ array of fixed size (kScratchBytes, about 0.9 MiB),
// which every GPU that loads the library holds until the process exits.
//
// The call synchronises the state's stream: it routes the draws on the
// host between its two kernels.
//
// Limits: states of at most 30 qubits (16384 chunks of 2^16 amplitudes) and
// at most 16384 shots per call; larger requests are refused.
//
// Sharing: every call on every state of a device uses the same array (and
// the same host staging arrays), and the array keeps the previous call's
// contents; the parts that must start at zero are cleared by each call.
// Calls that overlap — on the GPU or from several host threads — race.
#include <algorithm>

#include "zc_arith.cuh"
#include "zc_internal.h"
#include "zc_rng.h"

namespace zc {
namespace {

constexpr uint64_t kMaxChunks = 16384;  // 2^30 amplitudes in chunks of 2^16
constexpr uint64_t kMaxShots = 16384;
constexpr size_t kPartOff = 0;
constexpr size_t kDrawOff = kPartOff + kMaxChunks * sizeof(double);
constexpr size_t kOutOff = kDrawOff + kMaxShots * sizeof(double);
constexpr size_t kChunkOff = kOutOff + kMaxShots * sizeof(uint64_t);
constexpr size_t kScratchBytes = kChunkOff + kMaxShots * sizeof(SampleChunk);
constexpr int kMaxDevices = 64;

// The scratch: chunk masses | draws | indices | touched-chunk descriptors.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch per device (the host-side name is only a stand-in).
static unsigned char *g_scratch_addr[kMaxDevices];

// Host staging in static storage (no heap allocation).
static double h_part[kMaxChunks];
static double h_cum[kMaxChunks + 1];
static double h_us[kMaxShots];
static SampleChunk h_chunks[kMaxShots];

__device__ __forceinline__ double p2(double r, double i) { return radd(rmul(r, r), rmul(i, i)); }

// Chunk masses in the sampler's order (src/sample.rs:38-50): one serial f64
// chain per 2^16-element chunk; one thread per chunk, a warp stages 32
// chunks x 32 elements through shared memory to keep loads coalesced.
template <typename T>
__global__ void __launch_bounds__(64) k_masses_fixed(const T *__restrict__ re, const T *__restrict__ im,
                                                     uint64_t total, uint64_t chunk, uint64_t nchunks,
                                                     double *__restrict__ part) {
    __shared__ double sr[2][32][33];
    __shared__ double si[2][32][33];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint64_t c_base = ((uint64_t)blockIdx.x * 2 + warp) * 32;
    const uint64_t my_c = c_base + lane;
    double acc = 0.0;
    for (uint64_t off = 0; off < chunk; off += 32) {
        for (int row = 0; row < 32; row++) {
            const uint64_t c = c_base + row, e = off + lane;
            double vr = 0.0, vi = 0.0;
            if (c < nchunks && e < chunk && c * chunk + e < total) {
                vr = (double)re[c * chunk + e];
                vi = (double)im[c * chunk + e];
            }
            sr[warp][row][lane] = vr;
            si[warp][row][lane] = vi;
        }
        __syncwarp();
        if (my_c < nchunks) {
            const uint64_t lim = chunk - off < 32 ? chunk - off : 32;
            for (uint64_t e = 0; e < lim && my_c * chunk + off + e < total; e++)
                acc = radd(acc, p2(sr[warp][lane][e], si[warp][lane][e]));
        }
        __syncwarp();
    }
    if (my_c < nchunks) part[my_c] = acc;
}

// Per touched chunk, the serial rescan of src/sample.rs:64-108, one warp per
// chunk: the lanes load 32 consecutive amplitudes (coalesced) and square
// them; lane 0 adds the squares into the running f64 sum in index order and
// emits every draw below it, exactly as the serial loop does.
constexpr int kScanThreads = 128;

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_fixed(const T *__restrict__ re, const T *__restrict__ im,
                                                             const SampleChunk *__restrict__ cs, uint64_t ncs,
                                                             const double *__restrict__ us,
                                                             uint64_t *__restrict__ out, uint64_t chunk_len,
                                                             uint64_t total) {
    const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;  // warp-uniform
    const int lane = threadIdx.x % 32;
    if (w >= ncs) return;
    const SampleChunk sc = cs[w];
    const uint64_t lo = sc.chunk * chunk_len, hi = lo + chunk_len < total ? lo + chunk_len : total;
    uint64_t ptr = sc.s0;  // lane 0's cursor
    double acc = sc.cum;
    double u = ptr < sc.s1 ? us[ptr] : 0.0;
    int done = ptr >= sc.s1;
    for (uint64_t base = lo; base < hi && !done; base += 32) {
        const uint64_t i = base + lane;
        const double v = i < hi ? p2((double)re[i], (double)im[i]) : 0.0;
        for (int e = 0; e < 32; e++) {
            const double x = __shfl_sync(0xffffffffu, v, e);
            if (lane == 0 && !done && base + e < hi) {
                acc = radd(acc, x);
                while (u < acc) {
                    out[ptr++] = base + e;
                    if (ptr == sc.s1) {
                        done = 1;
                        break;
                    }
                    u = us[ptr];
                }
            }
        }
        done = __shfl_sync(0xffffffffu, done, 0);
    }
    const uint64_t left = __shfl_sync(0xffffffffu, ptr, 0);
    if (left < sc.s1) {  // leftover draws go to the chunk's last nonzero index
        uint64_t last_nz = hi - 1;
        for (uint64_t top = hi; top > lo; top = top > lo + 32 ? top - 32 : lo) {
            const bool in = top >= lo + 1 + (uint64_t)lane;
            const uint64_t i = in ? top - 1 - lane : lo;
            const unsigned m = __ballot_sync(0xffffffffu, in && p2((double)re[i], (double)im[i]) > 0.0);
            if (m) {  // the lowest set lane holds the highest index
                last_nz = top - 1 - (uint64_t)(__ffs(m) - 1);
                break;
            }
        }
        if (lane == 0)
            for (uint64_t k = left; k < sc.s1; k++) out[k] = last_nz;
    }
}

// Once per device, with that device current: resolve g_scratch's device address.
int scratch_for(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(ZC_ERR_UNSUPPORTED, "device ordinal beyond the scratch table");
    if (!g_scratch_addr[dev]) {
        int cur = -1;
        ZC_CUDA(cudaGetDevice(&cur));
        if (cur != dev)
            return fail(ZC_ERR_INVALID, "sample_noalloc: the state's device must be the current device");
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_scratch)");
        g_scratch_addr[dev] = (unsigned char *)p;
    }
    *out = g_scratch_addr[dev];
    return ZC_OK;
}

template <typename T>
int sample_fixed(zc_state *st, uint64_t shots, uint64_t seed, uint64_t *out, unsigned char *scratch) {
    const uint64_t chunk = st->len < (1ull << kSampleChunkLog2) ? st->len : (1ull << kSampleChunkLog2);
    const uint64_t nch = (st->len + chunk - 1) / chunk;
    double *d_part = (double *)(scratch + kPartOff);
    double *d_us = (double *)(scratch + kDrawOff);
    uint64_t *d_out = (uint64_t *)(scratch + kOutOff);
    SampleChunk *d_cs = (SampleChunk *)(scratch + kChunkOff);
    const T *re = (const T *)st->re, *im = (const T *)st->im;
    const int blocks = (int)((nch + 63) / 64);
    k_masses_fixed<T><<<blocks, 64, 0, st->stream>>>(re, im, st->len, chunk, nch, d_part);
    ZC_CUDA(cudaGetLastError());
    ZC_CUDA(cudaMemcpyAsync(h_part, d_part, nch * sizeof(double), cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    h_cum[0] = 0.0;
    for (uint64_t c = 0; c < nch; c++) h_cum[c + 1] = h_cum[c] + h_part[c];
    const double total = h_cum[nch];
    Xoshiro rng(seed);
    for (uint64_t i = 0; i < shots; i++) h_us[i] = rng.f64() * total;
    std::sort(h_us, h_us + shots);
    uint64_t ntouched = 0;
    uint64_t prev = std::lower_bound(h_us, h_us + shots, h_cum[0]) - h_us;
    for (uint64_t c = 0; c < nch; c++) {
        const uint64_t next = std::lower_bound(h_us, h_us + shots, h_cum[c + 1]) - h_us;
        if (prev < next) h_chunks[ntouched++] = SampleChunk{c, prev, next, h_cum[c]};
        prev = next;
    }
    ZC_CUDA(cudaMemcpyAsync(d_us, h_us, shots * sizeof(double), cudaMemcpyHostToDevice, st->stream));
    ZC_CUDA(cudaMemsetAsync(d_out, 0, shots * sizeof(uint64_t), st->stream));  // unresolved draws read 0
    if (ntouched) {
        ZC_CUDA(cudaMemcpyAsync(d_cs, h_chunks, ntouched * sizeof(SampleChunk), cudaMemcpyHostToDevice, st->stream));
        const uint64_t warps_per_cta = kScanThreads / 32;
        k_scan_fixed<T><<<(int)((ntouched + warps_per_cta - 1) / warps_per_cta), kScanThreads, 0, st->stream>>>(
            re, im, d_cs, ntouched, d_us, d_out, chunk, st->len);
        ZC_CUDA(cudaGetLastError());
    }
    ZC_CUDA(cudaMemcpyAsync(out, d_out, shots * sizeof(uint64_t), cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    return check_device_error(st);  // as zc_sample: a kernel that gave up left a wrong state
}

}  // namespace
}  // namespace zc

using namespace zc;

extern "C" int zc_sample_noalloc(zc_state *st, uint64_t shots, uint64_t seed, uint64_t *out) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    if (shots == 0) return ZC_OK;
    if (!out) return fail(ZC_ERR_INVALID, "sample_noalloc: null output");
    if (!st->queue.empty())
        return fail(ZC_ERR_INVALID, "sample_noalloc: ops are still queued; call zc_finish first");
    if (shots > kMaxShots) return fail(ZC_ERR_INVALID, "sample_noalloc: at most 16384 shots per call");
    if (st->len > kMaxChunks * (1ull << kSampleChunkLog2))
        return fail(ZC_ERR_INVALID, "sample_noalloc: at most 30 qubits (16384 chunks of 2^16 amplitudes)");
    unsigned char *scratch = nullptr;
    int rc = scratch_for(st->device, &scratch);
    if (rc) return rc;
    return st->prec == 64 ? sample_fixed<double>(st, shots, seed, out, scratch)
                          : sample_fixed<float>(st, shots, seed, out, scratch);
}
