// f64 reductions over the state (norm, prob_one, sampler chunk masses) and
// the sampler's per-chunk resolution pass.
//
// Exact mode keeps the reference's summation order: a serial f64 chain
// inside each 2^16-element chunk (src/sample.rs:38-50, src/state.rs:143-156),
// chunk partials combined serially in chunk order, so norm_sqr, prob_one and
// every sampled index are bit-identical to the CPU oracle for the same state
// bits. A dependent f64 add costs ~64 cycles on GB300 and the FP64 pipe
// issues one warp instruction per ~19 cycles per SM, so the chains are
// warp-specialised: seven producer warps load amplitudes and compute
// |a|^2 = r*r + i*i into a shared-memory ring (all lanes busy, loads
// batched), and one consumer warp runs 32 chains, one per lane, at one
// dependent add per element. The sampler's rescan records each chain's value
// at every 32-element stage boundary; draws then resolve in parallel by a
// binary search over those values and a replay of one stage, which repeats
// the chain's own additions bit for bit.
#include <atomic>

#include "zc_arith.cuh"
#include "zc_internal.h"

namespace zc {
namespace {

// |a|^2 in f64 exactly as `r * r + im * im` after widening (no FMA).
__device__ __forceinline__ double p2(double r, double i) { return radd(rmul(r, r), rmul(i, i)); }

// Non-negative doubles order like their IEEE bit patterns.
__device__ __forceinline__ unsigned long long dkey(double x) { return (unsigned long long)__double_as_longlong(x); }

// Named-barrier wait / arrive (non-.aligned forms: safe after divergence).
__device__ __forceinline__ void nb_sync(int id, int count) {
    asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void nb_arrive(int id, int count) {
    asm volatile("barrier.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

constexpr int kChainProducers = 7;  // producer warps; producer p owns ring slot p
constexpr int kChainThreads = 32 * (kChainProducers + 1);
constexpr int kStageElems = 32;     // elements per chain per stage
constexpr int kRowPad = kStageElems + 1;
constexpr size_t kChainSmem = (size_t)kChainProducers * 32 * kRowPad * sizeof(double);

// Named barriers: FULL(p) = 1 + p (producer p arrives, consumer waits),
// EMPTY(p) = 1 + kChainProducers + p (consumer arrives, producer p waits).
__device__ __forceinline__ int bar_full(int p) { return 1 + p; }
__device__ __forceinline__ int bar_empty(int p) { return 1 + kChainProducers + p; }

// Up to 32 serial chains per CTA (row r = consumer lane r).
// SCAN = false: rows are chunks blockIdx.x*32 + r of the index space (mode 0:
//   index h; mode 1, prob_one of qubit q: insert_zero(h, q) + 2^q); the final
//   chain value goes to part[row].
// SCAN = true: rows are the touched chunks cs[...]; a chain starts at the
//   chunk's cum_before and stops (for all rows together) once every row
//   exceeded its largest draw or ran out; rec[row][stage] holds the chain
//   value at each stage start, rec_nst[row] the stages run and rec_last[row]
//   1 + the last element with nonzero mass (0: none).
template <typename T, bool SCAN>
__global__ void __launch_bounds__(kChainThreads) k_chain(const T *__restrict__ re, const T *__restrict__ im,
                                                         uint64_t total, uint64_t chunk, uint64_t nrows, int mode,
                                                         uint32_t q, const SampleChunk *__restrict__ cs,
                                                         const double *__restrict__ us, double *__restrict__ part,
                                                         double *__restrict__ rec, uint32_t *__restrict__ rec_nst,
                                                         unsigned long long *__restrict__ rec_last,
                                                         uint32_t rec_stride) {
    extern __shared__ double ring[];  // [kChainProducers][32][kRowPad]
    __shared__ uint64_t s_first[32], s_len[32];
    __shared__ volatile int s_done;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint64_t row0 = (uint64_t)blockIdx.x * 32;
    const int R = nrows - row0 < 32 ? (int)(nrows - row0) : 32;
    if (warp == 0) {
        uint64_t first = 0, len = 0;
        if (lane < R) {
            const uint64_t c = SCAN ? cs[row0 + lane].chunk : row0 + lane;
            first = c * chunk;
            len = total - first < chunk ? total - first : chunk;
        }
        s_first[lane] = first;
        s_len[lane] = len;
        if (lane == 0) s_done = 0;
    }
    __syncthreads();
    uint64_t maxlen = 0;
    for (int r = 0; r < R; r++) maxlen = s_len[r] > maxlen ? s_len[r] : maxlen;
    const uint32_t nst = (uint32_t)((maxlen + kStageElems - 1) / kStageElems);
    const uint64_t sbit = 1ull << q;
    if (warp > 0) {
        const int p = warp - 1;
        double *buf = ring + (size_t)p * 32 * kRowPad;
        for (uint32_t s = p; s < nst; s += kChainProducers) {
            if (s >= (uint32_t)kChainProducers) nb_sync(bar_empty(p), 64);
            if (!s_done) {
                const uint64_t e = (uint64_t)s * kStageElems + lane;
                for (int r0 = 0; r0 < R; r0 += 8) {
                    T vr[8], vi[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        const int r = r0 + u;
                        vr[u] = vi[u] = (T)0;
                        if (r < R && e < s_len[r]) {
                            const uint64_t h = s_first[r] + e;
                            const uint64_t idx = mode == 0 ? h : insert_zero(h, q) + sbit;
                            vr[u] = re[idx];
                            vi[u] = im[idx];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 8; u++)
                        if (r0 + u < R) buf[(r0 + u) * kRowPad + lane] = p2(widen(vr[u]), widen(vi[u]));
                }
            }
            nb_arrive(bar_full(p), 64);
        }
        return;
    }
    // consumer warp: lane r runs row r's chain
    double acc = 0.0;
    unsigned long long stop = ~0ull, last = 0;
    if (SCAN && lane < R) {
        const SampleChunk sc = cs[row0 + lane];
        acc = sc.cum;
        stop = dkey(us[sc.s1 - 1]);
    }
    const uint64_t my_len = lane < R ? s_len[lane] : 0;
    bool all_done = false;
    uint32_t ran = nst;
    for (uint32_t s = 0; s < nst; s++) {
        const int p = (int)(s % kChainProducers);
        nb_sync(bar_full(p), 64);
        if (!all_done) {
            if (lane < R) {
                if (SCAN) rec[(row0 + lane) * rec_stride + s] = acc;
                const double *row = ring + ((size_t)p * 32 + lane) * kRowPad;
#pragma unroll 8
                for (int e = 0; e < kStageElems; e++) {
                    const double v = row[e];
                    acc = radd(acc, v);
                    if (SCAN && dkey(v) != 0ull) last = (unsigned long long)s * kStageElems + e + 1;
                }
            }
            const bool mine = lane >= R || (uint64_t)(s + 1) * kStageElems >= my_len || (SCAN && dkey(acc) > stop);
            if (__all_sync(0xffffffffu, mine)) {
                all_done = true;
                ran = s + 1;
                if (lane == 0) s_done = 1;
            }
        }
        if (s + kChainProducers < nst) nb_arrive(bar_empty(p), 64);
    }
    if (lane < R) {
        if (SCAN) {
            const uint32_t full = (uint32_t)((my_len + kStageElems - 1) / kStageElems);
            rec_nst[row0 + lane] = ran < full ? ran : full;
            rec_last[row0 + lane] = last;
        } else {
            part[row0 + lane] = acc;
        }
    }
}

__global__ void k_serial_sum(const double *__restrict__ part, uint64_t n, double *out) {
    double acc = 0.0;
    for (uint64_t i = 0; i < n; i++) acc = radd(acc, part[i]);
    *out = acc;
}

// Sampler pass 2 resolution (src/sample.rs:64-108), one CTA per touched
// chunk, one thread per draw: the draw lands in the last stage t whose start
// value is <= u; replaying stage t's additions from that value gives the
// first index i with u < acc_i, the index the serial rescan emits. A draw
// never exceeded by the chain goes to the chunk's last index with nonzero
// mass (its last index if none).
template <typename T>
__global__ void __launch_bounds__(128) k_resolve(const T *__restrict__ re, const T *__restrict__ im,
                                                 const SampleChunk *__restrict__ cs, const double *__restrict__ us,
                                                 uint64_t *__restrict__ out, uint64_t chunk_len, uint64_t total,
                                                 const double *__restrict__ rec, const uint32_t *__restrict__ rec_nst,
                                                 const unsigned long long *__restrict__ rec_last,
                                                 uint32_t rec_stride) {
    const uint64_t b = blockIdx.x;
    const SampleChunk sc = cs[b];
    const uint64_t first = sc.chunk * chunk_len;
    const uint64_t len = total - first < chunk_len ? total - first : chunk_len;
    const uint32_t n = rec_nst[b];
    const double *A = rec + b * rec_stride;
    for (uint64_t d = sc.s0 + threadIdx.x; d < sc.s1; d += blockDim.x) {
        const unsigned long long uk = dkey(us[d]);
        uint32_t lo = 0, hi = n - 1;  // A[0] = cum_before <= u by the host's routing
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (dkey(A[mid]) <= uk) lo = mid;
            else hi = mid - 1;
        }
        double acc = A[lo];
        const uint64_t e0 = (uint64_t)lo * kStageElems;
        const uint64_t e1 = e0 + kStageElems < len ? e0 + kStageElems : len;
        uint64_t res = ~0ull;
        for (uint64_t e = e0; e < e1; e++) {
            acc = radd(acc, p2(widen(re[first + e]), widen(im[first + e])));
            if (uk < dkey(acc)) {
                res = first + e;
                break;
            }
        }
        if (res == ~0ull) res = rec_last[b] ? first + rec_last[b] - 1 : first + len - 1;
        out[d] = res;
    }
}

// ------------------------------------------------------------------
// Fast mode (ZC_FLAG_FAST): the same quantities as parallel double-float
// reductions on the FP32 pipe (~2^-46 relative error per step instead of
// the reference's serial f64 order). Chunk boundaries and the host routing
// of draws are the exact path's; only the order of additions inside a
// chunk differs, so a draw can move by one index only where it falls
// within rounding distance of a cumulative boundary.

// a + b in double-float (TwoSum on the high parts, low parts summed).
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    float e;
    const float s = two_sum(a.x, b.x, e);
    return df_norm(s, __fadd_rn(e, __fadd_rn(a.y, b.y)));
}

__device__ __forceinline__ float2 p2_df(double r, double i) {
    const float2 a = df_from_f64(r), b = df_from_f64(i);
    return df_dot2(a, a, b, b);
}

__device__ __forceinline__ float2 p2_df(float r, float i) {
    const float2 a = make_float2(r, 0.f), b = make_float2(i, 0.f);
    return df_dot2(a, a, b, b);
}

__device__ __forceinline__ float2 shfl_xor_df(float2 v, int m) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

__device__ __forceinline__ float2 shfl_up_df(float2 v, int d) {
    return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
}

// Non-negative value as an order-preserving integer key (IEEE bits of f64).
__device__ __forceinline__ unsigned long long df_key(float2 v) {
    return (unsigned long long)__double_as_longlong(df_to_f64(v));
}

constexpr int kDfThreads = 256;

// CTA-wide double-float sum; every thread gets the result. `red` holds 8 slots.
__device__ __forceinline__ float2 block_sum_df(float2 v, float2 *red) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v = df_add(v, shfl_xor_df(v, m));
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    float2 t = make_float2(0.f, 0.f);
    for (int w = 0; w < (int)(blockDim.x / 32); w++) t = df_add(t, red[w]);
    return t;
}

// One CTA per chunk (mode and index map as k_chunk_sums); f64 partials.
template <typename T>
__global__ void __launch_bounds__(kDfThreads) k_chunk_sums_df(const T *__restrict__ re, const T *__restrict__ im,
                                                              uint64_t total, uint64_t chunk, int mode, uint32_t q,
                                                              double *__restrict__ part) {
    __shared__ float2 red[kDfThreads / 32];
    const uint64_t lo = (uint64_t)blockIdx.x * chunk;
    const uint64_t hi = lo + chunk < total ? lo + chunk : total;
    const uint64_t s = 1ull << q;
    float2 acc[4] = {};
    for (uint64_t h0 = lo + threadIdx.x; h0 < hi; h0 += 4 * kDfThreads) {
        T vr[4], vi[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint64_t h = h0 + (uint64_t)u * kDfThreads;
            vr[u] = vi[u] = (T)0;
            if (h < hi) {
                const uint64_t idx = mode == 0 ? h : insert_zero(h, q) + s;
                vr[u] = re[idx];
                vi[u] = im[idx];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; u++) acc[u] = df_add(acc[u], p2_df(vr[u], vi[u]));
    }
    const float2 t = block_sum_df(df_add(df_add(acc[0], acc[1]), df_add(acc[2], acc[3])), red);
    if (threadIdx.x == 0) part[blockIdx.x] = df_to_f64(t);
}

// Sum of n f64 partials into *out (one CTA).
__global__ void __launch_bounds__(kDfThreads) k_sum_df(const double *__restrict__ part, uint64_t n, double *out) {
    __shared__ float2 red[kDfThreads / 32];
    float2 acc = make_float2(0.f, 0.f);
    for (uint64_t i = threadIdx.x; i < n; i += kDfThreads) acc = df_add(acc, df_from_f64(part[i]));
    const float2 t = block_sum_df(acc, red);
    if (threadIdx.x == 0) *out = df_to_f64(t);
}

// Sampler pass 2, one CTA per touched chunk: tiles of 2048 elements get a
// CTA-wide inclusive prefix of |a|^2 (double-float) on top of the running
// cumulative; each draw of the tile resolves by binary search to the first
// index whose cumulative exceeds it (the reference's `us[ptr] < acc`).
// Draws left over past the chunk go to its last nonzero index.
constexpr int kScanPer = 8;
constexpr int kScanTile = kDfThreads * kScanPer;

template <typename T>
__global__ void __launch_bounds__(kDfThreads) k_sample_scan_df(const T *__restrict__ re, const T *__restrict__ im,
                                                               const SampleChunk *__restrict__ cs,
                                                               const double *__restrict__ us,
                                                               uint64_t *__restrict__ out, uint64_t chunk_len,
                                                               uint64_t total) {
    __shared__ float2 s_cum[kScanTile];
    __shared__ float2 s_wsum[kDfThreads / 32];
    __shared__ unsigned long long s_last;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const SampleChunk sc = cs[blockIdx.x];
    const uint64_t lo = sc.chunk * chunk_len;
    const uint64_t hi = lo + chunk_len < total ? lo + chunk_len : total;
    uint64_t ptr = sc.s0;
    float2 base = df_from_f64(sc.cum);  // truncated: never above the host's cum
    unsigned long long my_last = 0;     // 1 + last index with nonzero mass seen
    for (uint64_t t0 = lo; t0 < hi && ptr < sc.s1; t0 += kScanTile) {
        const uint64_t e0 = t0 + (uint64_t)tid * kScanPer;
        float2 pre[kScanPer];
        float2 run = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < kScanPer; j++) {
            const uint64_t i = e0 + j;
            float2 p = make_float2(0.f, 0.f);
            if (i < hi) {
                p = p2_df(re[i], im[i]);
                if (p.x > 0.f) my_last = i + 1;
            }
            run = df_add(run, p);
            pre[j] = run;
        }
        float2 incl = run;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const float2 v = shfl_up_df(incl, d);
            if (lane >= d) incl = df_add(v, incl);
        }
        float2 excl = shfl_up_df(incl, 1);
        if (lane == 0) excl = make_float2(0.f, 0.f);
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        float2 wpre = make_float2(0.f, 0.f);
        for (int w = 0; w < warp; w++) wpre = df_add(wpre, s_wsum[w]);
        const float2 tb = df_add(base, df_add(wpre, excl));
#pragma unroll
        for (int j = 0; j < kScanPer; j++) s_cum[tid * kScanPer + j] = df_add(tb, pre[j]);
        __syncthreads();
        const int nvalid = hi - t0 < (uint64_t)kScanTile ? (int)(hi - t0) : kScanTile;
        const unsigned long long end_key = df_key(s_cum[nvalid - 1]);
        uint64_t resolved = 0;
        for (uint64_t d0 = ptr; d0 < sc.s1; d0 += kDfThreads) {
            const uint64_t d = d0 + tid;
            int in = 0;
            if (d < sc.s1) {
                const unsigned long long uk = (unsigned long long)__double_as_longlong(us[d]);
                if (uk < end_key) {
                    in = 1;
                    int a = 0, b = nvalid - 1;  // first j with key(cum_j) > u; j = nvalid-1 qualifies
                    while (a < b) {
                        const int m = (a + b) / 2;
                        if (df_key(s_cum[m]) > uk) b = m;
                        else a = m + 1;
                    }
                    out[d] = t0 + (uint64_t)a;
                }
            }
            const int cnt = __syncthreads_count(in);
            resolved += (uint64_t)cnt;
            if (cnt < kDfThreads) break;
        }
        ptr += resolved;
        base = s_cum[nvalid - 1];
        __syncthreads();  // s_cum and s_wsum are rewritten by the next tile
    }
    if (ptr < sc.s1) {
        if (tid == 0) s_last = 0;
        __syncthreads();
        if (my_last) atomicMax(&s_last, my_last);
        __syncthreads();
        const uint64_t ln = s_last ? s_last - 1 : hi - 1;
        for (uint64_t d = ptr + tid; d < sc.s1; d += kDfThreads) out[d] = ln;
    }
}

// Launch k_chain (the exact chunk chains); rec != nullptr selects SCAN.
template <typename T, bool SCAN>
int run_chain(zc_state *st, unsigned blocks, uint64_t total, uint64_t chunk, uint64_t nrows, int mode, uint32_t q,
              const SampleChunk *cs, const double *us, double *part, double *rec, uint32_t stride) {
    static std::atomic<bool> attr{false};  // set once per process; racing first calls repeat it
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_chain<T, SCAN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kChainSmem));
        attr = true;
    }
    unsigned long long *rec_last = nullptr;
    uint32_t *rec_nst = nullptr;
    if (SCAN) {
        rec_last = (unsigned long long *)(rec + nrows * stride);
        rec_nst = (uint32_t *)(rec_last + nrows);
    }
    k_chain<T, SCAN><<<blocks, kChainThreads, kChainSmem, st->stream>>>(
        (const T *)st->re, (const T *)st->im, total, chunk, nrows, mode, q, cs, us, part, rec, rec_nst, rec_last,
        stride);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

}  // namespace

int launch_chunk_sums(zc_state *st, int mode, uint32_t q, size_t *nchunks_out, bool exact, double *out) {
    const uint64_t total = mode == 0 ? st->len : st->len / 2;
    const uint64_t chunk = total < (1ull << kSampleChunkLog2) ? total : (1ull << kSampleChunkLog2);
    const uint64_t nch = (total + chunk - 1) / chunk;
    if (!out && nch > st->part_cap) {
        if (st->d_part) cudaFree(st->d_part);
        st->d_part = nullptr;
        ZC_CUDA(cudaMalloc(&st->d_part, nch * sizeof(double)));
        st->part_cap = nch;
    }
    double *part = out ? out : st->d_part;
    ProfScope ps(st, K_CHUNK_SUMS, (mode == 0 ? 1.0 : 0.5) * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    *nchunks_out = nch;
    if (!exact) {
        if (st->prec == 64)
            k_chunk_sums_df<double><<<(unsigned)nch, kDfThreads, 0, st->stream>>>(
                (const double *)st->re, (const double *)st->im, total, chunk, mode, q, part);
        else
            k_chunk_sums_df<float><<<(unsigned)nch, kDfThreads, 0, st->stream>>>(
                (const float *)st->re, (const float *)st->im, total, chunk, mode, q, part);
        ZC_CUDA(cudaGetLastError());
        return ZC_OK;
    }
    const unsigned blocks = (unsigned)((nch + 31) / 32);
    if (st->prec == 64)
        return run_chain<double, false>(st, blocks, total, chunk, nch, mode, q, nullptr, nullptr, part, nullptr, 0);
    return run_chain<float, false>(st, blocks, total, chunk, nch, mode, q, nullptr, nullptr, part, nullptr, 0);
}

int launch_serial_sum(zc_state *st, size_t nchunks, bool exact) {
    ProfScope ps(st, K_SERIAL_SUM, 8.0 * nchunks);
    st->ctr.launches++;
    if (exact)
        k_serial_sum<<<1, 1, 0, st->stream>>>(st->d_part, nchunks, st->d_scalar);
    else
        k_sum_df<<<1, kDfThreads, 0, st->stream>>>(st->d_part, nchunks, st->d_scalar);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

int launch_sample_scan(zc_state *st, const SampleChunk *d_chunks, size_t nchunks, const double *d_us,
                       uint64_t *d_out, uint64_t chunk_len, bool exact, void *d_scratch) {
    if (nchunks == 0) return ZC_OK;
    ProfScope ps(st, K_SAMPLE_SCAN, (double)nchunks * chunk_len * (st->prec / 8) * 2);
    st->ctr.launches++;
    if (!exact) {
        if (st->prec == 64)
            k_sample_scan_df<double><<<(unsigned)nchunks, kDfThreads, 0, st->stream>>>(
                (const double *)st->re, (const double *)st->im, d_chunks, d_us, d_out, chunk_len, st->len);
        else
            k_sample_scan_df<float><<<(unsigned)nchunks, kDfThreads, 0, st->stream>>>(
                (const float *)st->re, (const float *)st->im, d_chunks, d_us, d_out, chunk_len, st->len);
        ZC_CUDA(cudaGetLastError());
        return ZC_OK;
    }
    const uint32_t stride = (uint32_t)((chunk_len + kStageElems - 1) / kStageElems);
    double *rec = (double *)d_scratch;
    unsigned long long *rec_last = (unsigned long long *)(rec + nchunks * stride);
    uint32_t *rec_nst = (uint32_t *)(rec_last + nchunks);
    const unsigned blocks = (unsigned)((nchunks + 31) / 32);
    int rc = st->prec == 64 ? run_chain<double, true>(st, blocks, st->len, chunk_len, nchunks, 0, 0, d_chunks, d_us,
                                                      nullptr, rec, stride)
                            : run_chain<float, true>(st, blocks, st->len, chunk_len, nchunks, 0, 0, d_chunks, d_us,
                                                     nullptr, rec, stride);
    if (rc) return rc;
    if (st->prec == 64)
        k_resolve<double><<<(unsigned)nchunks, 128, 0, st->stream>>>((const double *)st->re, (const double *)st->im,
                                                                     d_chunks, d_us, d_out, chunk_len, st->len, rec,
                                                                     rec_nst, rec_last, stride);
    else
        k_resolve<float><<<(unsigned)nchunks, 128, 0, st->stream>>>((const float *)st->re, (const float *)st->im,
                                                                    d_chunks, d_us, d_out, chunk_len, st->len, rec,
                                                                    rec_nst, rec_last, stride);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

size_t sample_scan_scratch(size_t nchunks, uint64_t chunk_len, bool exact) {
    if (!exact) return 0;
    const size_t stride = (chunk_len + kStageElems - 1) / kStageElems;
    return nchunks * (stride * sizeof(double) + sizeof(unsigned long long) + sizeof(uint32_t)) + 256;
}

}  // namespace zc
