// f64 reductions over the state (norm, prob_one, sampler chunk masses) and
// the sampler's per-chunk resolution pass.
//
// The summation order is the reference's: a serial f64 chain inside each
// 2^16-element chunk (src/sample.rs:38-50, src/state.rs:143-156), chunk
// partials combined serially in chunk order. That order makes norm_sqr,
// prob_one and every sampled index bit-identical to the CPU oracle for the
// same state bits. One thread owns one chunk; a warp stages 32 chunks x 32
// elements through shared memory so its global loads stay coalesced.
#include "zc_arith.cuh"
#include "zc_internal.h"

namespace zc {
namespace {

constexpr int kWarps = 2;  // warps per CTA; one chunk per thread
constexpr int kStage = 32; // elements per chunk staged per step

// |a|^2 in f64 exactly as `r * r + im * im` after widening (no FMA).
__device__ __forceinline__ double p2(double r, double i) { return radd(rmul(r, r), rmul(i, i)); }

// Partial sums. mode 0: element e of chunk c is index c*chunk + e.
// mode 1 (prob_one of qubit q): half-index h = c*chunk + e maps to the
// q=1 member insert_zero(h, q) + 2^q.
template <typename T>
__global__ void __launch_bounds__(kWarps * 32) k_chunk_sums(const T *__restrict__ re, const T *__restrict__ im,
                                                            uint64_t total, uint64_t chunk, uint64_t nchunks,
                                                            int mode, uint32_t q, double *__restrict__ part) {
    __shared__ double sr[kWarps][32][kStage + 1];
    __shared__ double si[kWarps][32][kStage + 1];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint64_t c_base = ((uint64_t)blockIdx.x * kWarps + warp) * 32;
    const uint64_t my_c = c_base + lane;
    double acc = 0.0;
    const uint64_t s = 1ull << q;
    for (uint64_t off = 0; off < chunk; off += kStage) {
        // cooperative load: row = chunk (c_base + row), col = element off + col
        for (int row = 0; row < 32; row++) {
            const uint64_t c = c_base + row;
            const uint64_t e = off + lane;
            double vr = 0.0, vi = 0.0;
            if (c < nchunks && e < chunk) {
                const uint64_t h = c * chunk + e;
                if (h < total) {
                    const uint64_t idx = mode == 0 ? h : insert_zero(h, q) + s;
                    vr = (double)re[idx];
                    vi = (double)im[idx];
                }
            }
            sr[warp][row][lane] = vr;
            si[warp][row][lane] = vi;
        }
        __syncwarp();
        if (my_c < nchunks) {
            const uint64_t lim = chunk - off < (uint64_t)kStage ? chunk - off : (uint64_t)kStage;
            for (uint64_t e = 0; e < lim; e++) {
                const uint64_t h = my_c * chunk + off + e;
                if (h >= total) break;
                acc = radd(acc, p2(sr[warp][lane][e], si[warp][lane][e]));
            }
        }
        __syncwarp();
    }
    if (my_c < nchunks) part[my_c] = acc;
}

__global__ void k_serial_sum(const double *__restrict__ part, uint64_t n, double *out) {
    double acc = 0.0;
    for (uint64_t i = 0; i < n; i++) acc = radd(acc, part[i]);
    *out = acc;
}

// Sampler pass 2 (src/sample.rs:64-108): each touched chunk is rescanned
// serially with a running cumulative; draw ptr resolves to index i while
// us[ptr] < acc. Unresolved draws land on the chunk's last index with
// nonzero probability.
template <typename T>
__global__ void k_sample_scan(const T *__restrict__ re, const T *__restrict__ im, const SampleChunk *__restrict__ cs,
                              uint64_t ncs, const double *__restrict__ us, uint64_t *__restrict__ out,
                              uint64_t chunk_len, uint64_t total) {
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= ncs) return;
    const SampleChunk sc = cs[t];
    const uint64_t lo = sc.chunk * chunk_len;
    const uint64_t hi = lo + chunk_len < total ? lo + chunk_len : total;
    uint64_t ptr = sc.s0;
    double acc = sc.cum;
    for (uint64_t i = lo; i < hi; i++) {
        acc = radd(acc, p2((double)re[i], (double)im[i]));
        while (ptr < sc.s1 && us[ptr] < acc) out[ptr++] = i;
        if (ptr == sc.s1) break;
    }
    if (ptr < sc.s1) {
        uint64_t last_nz = hi - 1;
        for (uint64_t i = hi; i-- > lo;) {
            if (p2((double)re[i], (double)im[i]) > 0.0) {
                last_nz = i;
                break;
            }
        }
        while (ptr < sc.s1) out[ptr++] = last_nz;
    }
}

}  // namespace

int launch_chunk_sums(zc_state *st, int mode, uint32_t q, size_t *nchunks_out) {
    const uint64_t total = mode == 0 ? st->len : st->len / 2;
    const uint64_t chunk = total < (1ull << kSampleChunkLog2) ? total : (1ull << kSampleChunkLog2);
    const uint64_t nch = (total + chunk - 1) / chunk;
    if (nch > st->part_cap) {
        if (st->d_part) cudaFree(st->d_part);
        st->d_part = nullptr;
        ZC_CUDA(cudaMalloc(&st->d_part, nch * sizeof(double)));
        st->part_cap = nch;
    }
    const uint64_t per_block = kWarps * 32;
    const int blocks = (int)((nch + per_block - 1) / per_block);
    ProfScope ps(st, K_CHUNK_SUMS, (mode == 0 ? 1.0 : 0.5) * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    if (st->prec == 64)
        k_chunk_sums<double><<<blocks, kWarps * 32, 0, st->stream>>>((const double *)st->re, (const double *)st->im,
                                                                     total, chunk, nch, mode, q, st->d_part);
    else
        k_chunk_sums<float><<<blocks, kWarps * 32, 0, st->stream>>>((const float *)st->re, (const float *)st->im,
                                                                    total, chunk, nch, mode, q, st->d_part);
    ZC_CUDA(cudaGetLastError());
    *nchunks_out = nch;
    return ZC_OK;
}

int launch_serial_sum(zc_state *st, size_t nchunks) {
    ProfScope ps(st, K_SERIAL_SUM, 8.0 * nchunks);
    st->ctr.launches++;
    k_serial_sum<<<1, 1, 0, st->stream>>>(st->d_part, nchunks, st->d_scalar);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

int launch_sample_scan(zc_state *st, const SampleChunk *d_chunks, size_t nchunks, const double *d_us,
                       uint64_t *d_out, uint64_t chunk_len) {
    if (nchunks == 0) return ZC_OK;
    ProfScope ps(st, K_SAMPLE_SCAN, (double)nchunks * chunk_len * (st->prec / 8) * 2);
    st->ctr.launches++;
    const int threads = 128;
    const int blocks = (int)((nchunks + threads - 1) / threads);
    if (st->prec == 64)
        k_sample_scan<double><<<blocks, threads, 0, st->stream>>>((const double *)st->re, (const double *)st->im,
                                                                  d_chunks, nchunks, d_us, d_out, chunk_len, st->len);
    else
        k_sample_scan<float><<<blocks, threads, 0, st->stream>>>((const float *)st->re, (const float *)st->im,
                                                                 d_chunks, nchunks, d_us, d_out, chunk_len, st->len);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

}  // namespace zc
