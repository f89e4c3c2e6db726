// Dense k-qubit blocks on tensor cores for f32 states (3xTF32).
//
// A fused block M (2^k x 2^k complex) acts on every group of 2^k amplitudes.
// In real form, with D = 2^k and R = 2D,
//     [Yr; Yi] = [[Mr, -Mi], [Mi, Mr]] . [Xr; Xi] = A' . X'
// is one real GEMM over the G = 2^(n-k) groups. Each product is split into
// TF32 parts, A = Ah + Al and X = Xh + Xl (Ah, Xh the TF32 roundings, Al, Xl
// the TF32 roundings of the remainders), and accumulated in FP32 as
// Ah.Xh + Ah.Xl + Al.Xh ("3xTF32"), close to FP32 accuracy on the TF32
// tensor pipe.
//
// k = 4..7 run on the 5th-generation tensor cores (k_block_umma): the GEMM
// is taken transposed, D[g][r] = sum_kk X'[kk][g] . A'[r][kk], so one
// tcgen05.mma covers M = 128 groups x N = R output rows x K = 8, with the
// FP32 accumulator tile (128 x R) in tensor memory. K is streamed in chunks
// of 32 through two shared-memory buffers: the A' chunk (pre-split and
// pre-laid-out on the host) arrives by one TMA bulk copy, the X' chunk is
// gathered, split and stored by all threads while the previous chunk's MMAs
// run. One thread issues the MMAs and commits them to an mbarrier; the
// epilogue reads the accumulator back with tcgen05.ld and scatters it.
// k = 3 (R = 16) uses warp-level mma.sync (k_block_tc).
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "zc_arith.cuh"
#include "zc_async.cuh"
#include "zc_internal.h"

namespace zc {
namespace {

constexpr int kTcThreads = 256;  // 8 warps
constexpr int kTcCols = 64;      // groups per CTA tile
constexpr int kTcSlice = 32;     // A' columns per shared-memory slice
constexpr int kTcPad = 4;        // row padding (floats) against bank conflicts

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float *d, const uint32_t *a, const uint32_t *b) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct TcParams {
    uint64_t groups;
    uint32_t k;
    uint32_t qs[kMaxUnitaryQubits];
    uint64_t offs[1 << kMaxUnitaryQubits];
};

// R = 2^(k+1). Shared memory: Xh, Xl [R][64 + pad], Ah, Al [R][32 + pad].
template <int R>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_block_tc(float *__restrict__ re, float *__restrict__ im, TcParams p, const float *__restrict__ ah_g,
               const float *__restrict__ al_g) {
    constexpr int D = R / 2;
    constexpr int SL = R < kTcSlice ? R : kTcSlice;  // A' columns per slice
    constexpr int LX = kTcCols + kTcPad, LA = SL + kTcPad;
    constexpr int MT = R / 16, NT = kTcCols / 8;
    constexpr int TILES = MT * NT;
    constexpr int TPW = TILES >= 8 ? TILES / 8 : 1;  // output tiles per warp
    extern __shared__ __align__(16) float sm[];
    float *xh = sm, *xl = xh + R * LX, *ah = xl + R * LX, *al = ah + R * LA;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const int gid = lane >> 2, tig = lane & 3;
    const uint64_t ntiles = (p.groups + kTcCols - 1) / kTcCols;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t g0 = tile * kTcCols;
        // gather X' = [Xr; Xi] for 64 groups, split into TF32 hi / lo
        for (int e = tid; e < D * kTcCols; e += blockDim.x) {
            const int c = e % kTcCols, j = e / kTcCols;
            float vr = 0.f, vi = 0.f;
            if (g0 + c < p.groups) {
                const uint64_t idx = insert_zeros(g0 + c, p.qs, (int)p.k) | p.offs[j];
                vr = re[idx];
                vi = im[idx];
            }
            const float hr = __uint_as_float(to_tf32(vr)), hi = __uint_as_float(to_tf32(vi));
            xh[j * LX + c] = hr;
            xl[j * LX + c] = __uint_as_float(to_tf32(vr - hr));
            xh[(D + j) * LX + c] = hi;
            xl[(D + j) * LX + c] = __uint_as_float(to_tf32(vi - hi));
        }
        float acc[TPW][4];
#pragma unroll
        for (int t = 0; t < TPW; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.f;
        for (int k0 = 0; k0 < R; k0 += SL) {
            __syncthreads();  // X' complete (first slice) / previous slice consumed
            for (int e = tid; e < R * SL; e += blockDim.x) {
                const int r = e / SL, c = e % SL;
                ah[r * LA + c] = ah_g[(size_t)r * R + k0 + c];
                al[r * LA + c] = al_g[(size_t)r * R + k0 + c];
            }
            __syncthreads();
            if (warp * TPW < TILES) {
#pragma unroll
                for (int kk = 0; kk < SL; kk += 8) {
#pragma unroll
                    for (int t = 0; t < TPW; t++) {
                        const int tidx = warp * TPW + t;
                        const int m = tidx / NT, n = tidx % NT;
                        const int r0 = m * 16 + gid, c0 = n * 8 + gid;
                        uint32_t a_hi[4], a_lo[4], b_hi[2], b_lo[2];
                        a_hi[0] = __float_as_uint(ah[r0 * LA + kk + tig]);
                        a_hi[1] = __float_as_uint(ah[(r0 + 8) * LA + kk + tig]);
                        a_hi[2] = __float_as_uint(ah[r0 * LA + kk + tig + 4]);
                        a_hi[3] = __float_as_uint(ah[(r0 + 8) * LA + kk + tig + 4]);
                        a_lo[0] = __float_as_uint(al[r0 * LA + kk + tig]);
                        a_lo[1] = __float_as_uint(al[(r0 + 8) * LA + kk + tig]);
                        a_lo[2] = __float_as_uint(al[r0 * LA + kk + tig + 4]);
                        a_lo[3] = __float_as_uint(al[(r0 + 8) * LA + kk + tig + 4]);
                        const int kr = k0 + kk + tig;
                        b_hi[0] = __float_as_uint(xh[kr * LX + c0]);
                        b_hi[1] = __float_as_uint(xh[(kr + 4) * LX + c0]);
                        b_lo[0] = __float_as_uint(xl[kr * LX + c0]);
                        b_lo[1] = __float_as_uint(xl[(kr + 4) * LX + c0]);
                        mma_tf32(acc[t], a_lo, b_hi);
                        mma_tf32(acc[t], a_hi, b_lo);
                        mma_tf32(acc[t], a_hi, b_hi);
                    }
                }
            }
        }
        __syncthreads();  // all reads of X' done: reuse xh for Y'
        if (warp * TPW < TILES) {
#pragma unroll
            for (int t = 0; t < TPW; t++) {
                const int tidx = warp * TPW + t;
                const int m = tidx / NT, n = tidx % NT;
                const int r0 = m * 16 + gid, c0 = n * 8 + 2 * tig;
                xh[r0 * LX + c0] = acc[t][0];
                xh[r0 * LX + c0 + 1] = acc[t][1];
                xh[(r0 + 8) * LX + c0] = acc[t][2];
                xh[(r0 + 8) * LX + c0 + 1] = acc[t][3];
            }
        }
        __syncthreads();
        for (int e = tid; e < D * kTcCols; e += blockDim.x) {
            const int c = e % kTcCols, j = e / kTcCols;
            if (g0 + c < p.groups) {
                const uint64_t idx = insert_zeros(g0 + c, p.qs, (int)p.k) | p.offs[j];
                re[idx] = xh[j * LX + c];
                im[idx] = xh[(D + j) * LX + c];
            }
        }
        __syncthreads();
    }
}

template <int R>
int run_tc(zc_state *st, const TcParams &p, const float *ah, const float *al) {
    constexpr int SL = R < kTcSlice ? R : kTcSlice;
    const size_t smem = (size_t)(2 * R * (kTcCols + kTcPad) + 2 * R * (SL + kTcPad)) * sizeof(float);
    static std::atomic<bool> attr{false};  // set once per process; racing first calls repeat it
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_block_tc<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    const uint64_t ntiles = (p.groups + kTcCols - 1) / kTcCols;
    const int blocks = (int)std::min<uint64_t>(ntiles, (uint64_t)st->num_sms);
    k_block_tc<R><<<blocks, kTcThreads, smem, st->stream>>>((float *)st->re, (float *)st->im, p, ah, al);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

// ------------------------------------------------------------------
// tcgen05 path (k = 4..7)

constexpr int kUmThreads = 256;
constexpr int kUmM = 128;                 // groups per tile (MMA M)
constexpr int kUmKc = 32;                 // K per chunk
constexpr uint32_t kUmSbo = 128;          // core-matrix (8 rows x 16 B) step along M / N
constexpr uint32_t kUmXLbo = kUmM * 16;   // core-matrix step along K in the X' chunk
constexpr uint32_t kUmXBytes = kUmM * kUmKc * 4;

// Shared-memory matrix descriptor, K-major, no swizzle: start address,
// leading (K) and stride (M/N) byte offsets between 8x16-byte core matrices.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor: FP32 accumulator, TF32 A and B, both K-major.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// A' on the device: [Ah | Al], each R x R floats laid out as the MMA's
// K-major B operand (byte offset of (r, kk) = (kk/4)*16R + (r/8)*128 +
// (r%8)*16 + (kk%4)*4), so K chunk c of either half is one contiguous run
// of 128R bytes. For R <= 128 the whole A' stays in shared memory; for
// R = 256 (512 KiB) its chunks stream through two buffers.
__host__ __device__ constexpr bool umma_resident(int R) { return R <= 128; }
__host__ __device__ constexpr size_t umma_smem_bytes(int R) {
    return 4 * (size_t)kUmXBytes + (umma_resident(R) ? 2 * (size_t)R * R * 4 : 4 * (size_t)R * kUmKc * 4);
}

template <int R>
__global__ void __launch_bounds__(kUmThreads, R <= 64 ? 2 : 1)
    k_block_umma(float *__restrict__ re, float *__restrict__ im, TcParams p, const float *__restrict__ a,
                 int *__restrict__ err) {
    constexpr bool RES = umma_resident(R);
    constexpr int D = R / 2;
    constexpr int NC = R / kUmKc;
    constexpr int kQ = kUmKc / 4 / (kUmThreads / kUmM);  // K quads a thread gathers per chunk
    constexpr int kV = 4 * kQ;                           // values a thread gathers per chunk
    constexpr uint32_t kBLbo = R * 16;
    constexpr uint32_t kAHalf = R * R * 4;               // bytes of Ah (or Al)
    constexpr uint32_t kBChunk = R * kUmKc * 4;          // bytes of one K chunk of Ah (or Al)
    constexpr uint32_t kIdesc = umma_idesc_tf32(kUmM, R);
    extern __shared__ __align__(1024) unsigned char smu[];
    __shared__ uint64_t load_bar[2], mma_bar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int s_fail;
    unsigned char *const xbuf0 = smu, *const abuf = smu + 4 * kUmXBytes;
    const int tid = threadIdx.x, warp = tid / 32;
    if (tid == 0) {
        for (int b = 0; b < 2; b++) {
            mbar_init(&load_bar[b], 1);
            mbar_init(&mma_bar[b], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(R));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmem_base;
    const uint64_t ntiles = (p.groups + kUmM - 1) / kUmM;
    const uint64_t my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    const uint64_t nsteps = my_tiles * NC;  // (tile, K chunk) steps of this CTA
    // A': all of it (resident) or the first chunk (streamed), by TMA
    if (tid == 0 && nsteps > 0) {
        if (RES) {
            mbar_expect_tx(&load_bar[0], 2 * kAHalf);
            bulk_load(abuf, a, kAHalf, &load_bar[0]);
            bulk_load(abuf + kAHalf, a + R * R, kAHalf, &load_bar[0]);
        } else {
            mbar_expect_tx(&load_bar[0], 2 * kBChunk);
            bulk_load(abuf, a, kBChunk, &load_bar[0]);
            bulk_load(abuf + kBChunk, a + R * R, kBChunk, &load_bar[0]);
        }
    }
    uint32_t load_phase[2] = {0, 0}, mma_phase[2] = {0, 0};
    int pending[2] = {0, 0};
    bool failed = false, a_ready = false;
    const int gl = tid % kUmM;     // this thread's group within a tile (gather and epilogue)
    const int quad0 = tid / kUmM;  // first K quad it gathers
    auto group_base = [&](uint64_t s, bool &valid) {
        const uint64_t g = (blockIdx.x + (s / NC) * gridDim.x) * kUmM + gl;
        valid = g < p.groups;
        return valid ? insert_zeros(g, p.qs, (int)p.k) : 0ull;
    };
    // X' values of step s (this thread's group, its K quads of the chunk)
    auto gather = [&](uint64_t s, float *v) {
        bool valid;
        const uint64_t base = group_base(s, valid);
        const int c = (int)(s % NC);
#pragma unroll
        for (int m = 0; m < kQ; m++)
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int kk = c * kUmKc + (quad0 + m * (kUmThreads / kUmM)) * 4 + i;
                const int j = kk < D ? kk : kk - D;
                v[m * 4 + i] = valid ? (kk < D ? re : im)[base | p.offs[j]] : 0.f;
            }
    };
    // One (tile, K chunk) step; `cur` holds its gathered values, the gather
    // of step s + 2 goes into `fut` and stays in flight across two steps.
    // Returns false when a wait ran out (all threads agree).
    auto step = [&](uint64_t s, const float *cur, float *fut) -> bool {
        if (s + 2 < nsteps) gather(s + 2, fut);
        const int c = (int)(s % NC), b = (int)(s & 1);
        // X' buffer b was last read by the MMAs of step s - 2
        int bad = 0;
        if (pending[b]) {
            bad = !mbar_wait(&mma_bar[b], mma_phase[b]);
            mma_phase[b] ^= 1;
            pending[b] = 0;
        }
        if (__syncthreads_or(bad | s_fail)) return false;
        unsigned char *xb = xbuf0 + b * 2 * kUmXBytes;
#pragma unroll
        for (int m = 0; m < kQ; m++) {
            float4 hi, lo;
            hi.x = __uint_as_float(to_tf32(cur[m * 4 + 0]));
            hi.y = __uint_as_float(to_tf32(cur[m * 4 + 1]));
            hi.z = __uint_as_float(to_tf32(cur[m * 4 + 2]));
            hi.w = __uint_as_float(to_tf32(cur[m * 4 + 3]));
            lo.x = __uint_as_float(to_tf32(cur[m * 4 + 0] - hi.x));
            lo.y = __uint_as_float(to_tf32(cur[m * 4 + 1] - hi.y));
            lo.z = __uint_as_float(to_tf32(cur[m * 4 + 2] - hi.z));
            lo.w = __uint_as_float(to_tf32(cur[m * 4 + 3] - hi.w));
            const uint32_t off = (quad0 + m * (kUmThreads / kUmM)) * kUmXLbo + (gl / 8) * kUmSbo + (gl % 8) * 16;
            *reinterpret_cast<float4 *>(xb + off) = hi;
            *reinterpret_cast<float4 *>(xb + kUmXBytes + off) = lo;
        }
        fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            const int ab = RES ? 0 : b;  // A' buffer (streamed: one per step parity)
            bool ok = true;
            if (!RES || !a_ready) {
                ok = mbar_wait(&load_bar[ab], load_phase[ab]);
                load_phase[ab] ^= 1;
                a_ready = true;
            }
            if (!ok) {
                s_fail = 1;
            } else {
                tc_fence_after();
                const uint32_t xa = smem_addr(xb);
                const uint32_t ah = smem_addr(abuf) + (RES ? (uint32_t)c * 8 * kBLbo : (uint32_t)b * 2 * kBChunk);
                const uint32_t al = ah + (RES ? kAHalf : kBChunk);
#pragma unroll
                for (int k8 = 0; k8 < kUmKc / 8; k8++) {
                    const uint64_t dxh = umma_desc(xa + k8 * 2 * kUmXLbo, kUmXLbo, kUmSbo);
                    const uint64_t dxl = umma_desc(xa + kUmXBytes + k8 * 2 * kUmXLbo, kUmXLbo, kUmSbo);
                    const uint64_t dah = umma_desc(ah + k8 * 2 * kBLbo, kBLbo, kUmSbo);
                    const uint64_t dal = umma_desc(al + k8 * 2 * kBLbo, kBLbo, kUmSbo);
                    umma_tf32(tbase, dxl, dah, kIdesc, (c | k8) != 0);
                    umma_tf32(tbase, dxh, dal, kIdesc, 1);
                    umma_tf32(tbase, dxh, dah, kIdesc, 1);
                }
            }
            umma_commit(&mma_bar[b]);  // arrives once the MMAs issued so far are done
            if (!RES && s + 1 < nsteps) {
                // next step's A' chunk goes into the other buffer once its last
                // reader (the MMAs of step s - 1) is done
                const int b1 = b ^ 1;
                if (pending[b1]) {
                    if (!mbar_wait(&mma_bar[b1], mma_phase[b1])) s_fail = 1;
                    mma_phase[b1] ^= 1;
                    pending[b1] = 0;
                }
                const int c1 = (int)((s + 1) % NC);
                unsigned char *dst = abuf + b1 * 2 * kBChunk;
                mbar_expect_tx(&load_bar[b1], 2 * kBChunk);
                bulk_load(dst, a + (size_t)c1 * R * kUmKc, kBChunk, &load_bar[b1]);
                bulk_load(dst + kBChunk, a + R * R + (size_t)c1 * R * kUmKc, kBChunk, &load_bar[b1]);
            }
        }
        pending[b] = 1;
        if (c == NC - 1) {
            // tile complete: wait for its last MMAs, read the accumulator out
            bad = 0;
            for (int bb = 0; bb < 2; bb++)
                if (pending[bb]) {
                    bad |= !mbar_wait(&mma_bar[bb], mma_phase[bb]);
                    mma_phase[bb] ^= 1;
                    pending[bb] = 0;
                }
            if (__syncthreads_or(bad | s_fail)) return false;
            tc_fence_after();
            bool valid;
            const uint64_t base = group_base(s, valid);
            const uint32_t lane_base = (uint32_t)(32 * (warp % 4)) << 16;
#pragma unroll 1
            for (int col0 = (warp / 4) * (R / 2); col0 < (warp / 4 + 1) * (R / 2); col0 += 16) {
                uint32_t v[16];
                tmem_ld16(tbase + lane_base + (uint32_t)col0, v);
                if (valid) {
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        const int r = col0 + i;
                        const int j = r < D ? r : r - D;
                        (r < D ? re : im)[base | p.offs[j]] = __uint_as_float(v[i]);
                    }
                }
            }
            tc_fence_before();
            __syncthreads();  // accumulator read out before the next tile's MMAs overwrite it
        }
        return true;
    };
    // three register sets rotate roles (no copies of values still in flight)
    float va[kV], vb[kV], vc[kV];
    if (nsteps > 0) gather(0, va);
    if (nsteps > 1) gather(1, vb);
    for (uint64_t s = 0; s < nsteps && !failed; s += 3) {
        if (!step(s, va, vc)) failed = true;
        else if (s + 1 < nsteps && !step(s + 1, vb, va)) failed = true;
        else if (s + 2 < nsteps && !step(s + 2, vc, vb)) failed = true;
    }
    if (failed) {
        // let outstanding MMAs and copies finish (bounded) before the tensor memory goes
        for (int b = 0; b < 2; b++)
            if (pending[b]) mbar_wait(&mma_bar[b], mma_phase[b]);
        if (tid == 0) atomicExch(err, 3);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(R));
}

template <int R>
int run_umma(zc_state *st, const TcParams &p, const float *a) {
    constexpr size_t smem = umma_smem_bytes(R);
    static std::atomic<bool> attr{false};  // set once per process; racing first calls repeat it
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_block_umma<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    // resident CTAs per SM (shared memory, registers and tensor memory
    // decide), found once per process
    static std::atomic<int> cached_per_sm{0};
    int per_sm = cached_per_sm.load();
    if (!per_sm) {
        ZC_CUDA(cudaFuncSetAttribute(k_block_umma<R>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared));
        cudaFuncAttributes fa;
        ZC_CUDA(cudaFuncGetAttributes(&fa, k_block_umma<R>));
        int smem_sm = 0, regs_sm = 0;
        ZC_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, st->device));
        ZC_CUDA(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, st->device));
        const size_t per_cta_smem = smem + fa.sharedSizeBytes + 1024;  // + static + per-CTA reservation
        const int by_smem = (int)(smem_sm / per_cta_smem);
        const int by_regs = regs_sm / std::max(1, fa.numRegs * kUmThreads);
        per_sm = std::min(std::min(by_smem, by_regs), 512 / R);
        if (per_sm < 1) return fail(ZC_ERR_UNSUPPORTED, "tensor-core block kernel does not fit on an SM");
        cached_per_sm.store(per_sm);
    }
    const uint64_t ntiles = (p.groups + kUmM - 1) / kUmM;
    const int blocks = (int)std::min<uint64_t>(ntiles, (uint64_t)st->num_sms * per_sm);
    k_block_umma<R><<<blocks, kUmThreads, smem, st->stream>>>((float *)st->re, (float *)st->im, p, a, st->d_err);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

}  // namespace

// Round to TF32 (nearest, ties away from zero: the rounding of cvt.rna.tf32).
static float tf32_rna(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
    float r;
    memcpy(&r, &u, 4);
    return r;
}

// Entry (r, kk) of the real form A' = [[Mr, -Mi], [Mi, Mr]].
static double real_form(const double *mat, size_t D, size_t r, size_t kk) {
    const size_t i = r % D, j = kk % D;
    const double mr = mat[2 * (i * D + j)], mi = mat[2 * (i * D + j) + 1];
    return (r < D) == (kk < D) ? mr : (r < D ? -mi : mi);
}

int launch_block_tc(zc_state *st, const uint32_t *qs, uint32_t k, const double *mat) {
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * 4 * 2;
    if (st->prec != 32) return fail(ZC_ERR_UNSUPPORTED, "tensor-core blocks run on f32 states");
    if (k < 3 || k > 7) return fail(ZC_ERR_INVALID, "tensor-core blocks need k in 3..7");
    TcParams p{};
    p.k = k;
    p.groups = st->len >> k;
    for (uint32_t i = 0; i < k; i++) p.qs[i] = qs[i];
    for (uint32_t j = 0; j < (1u << k); j++) {
        uint64_t o = 0;
        for (uint32_t b = 0; b < k; b++)
            if ((j >> b) & 1) o |= 1ull << qs[b];
        p.offs[j] = o;
    }
    const size_t D = (size_t)1 << k, R = 2 * D;
    std::vector<float> a(2 * R * R);
    const void *dev = nullptr;
    if (k == 3) {
        // mma.sync path: [Ah | Al], row-major
        for (size_t r = 0; r < R; r++)
            for (size_t kk = 0; kk < R; kk++) {
                const double v = real_form(mat, D, r, kk);
                const float h = tf32_rna((float)v);
                a[r * R + kk] = h;
                a[R * R + r * R + kk] = tf32_rna((float)(v - (double)h));
            }
        int rc = arena_put(st, a.data(), a.size() * sizeof(float), &dev);
        if (rc) return rc;
        ProfScope ps(st, K_TC, 2.0 * st->len * 4 * 2);
        return run_tc<16>(st, p, (const float *)dev, (const float *)dev + R * R);
    }
    // tcgen05 path: [Ah | Al], each in the K-major B-operand layout
    for (size_t r = 0; r < R; r++)
        for (size_t kk = 0; kk < R; kk++) {
            const double v = real_form(mat, D, r, kk);
            const float h = tf32_rna((float)v);
            const size_t off = ((kk / 4) * (R * 16) + (r / 8) * 128 + (r % 8) * 16 + (kk % 4) * 4) / 4;
            a[off] = h;
            a[R * R + off] = tf32_rna((float)(v - (double)h));
        }
    int rc = arena_put(st, a.data(), a.size() * sizeof(float), &dev);
    if (rc) return rc;
    ProfScope ps(st, K_TC, 2.0 * st->len * 4 * 2);
    const float *ad = (const float *)dev;
    switch (k) {
        case 4: return run_umma<32>(st, p, ad);
        case 5: return run_umma<64>(st, p, ad);
        case 6: return run_umma<128>(st, p, ad);
        default: return run_umma<256>(st, p, ad);
    }
}

}  // namespace zc
