// Dense k-qubit blocks on tensor cores for f32 states (3xTF32).
//
// A fused block M (2^k x 2^k complex, k = 3..7) acts on every group of 2^k
// amplitudes. In real form, with D = 2^k and R = 2D,
//     [Yr; Yi] = [[Mr, -Mi], [Mi, Mr]] . [Xr; Xi]
// is one real GEMM A' (R x R) . X' (R x G) over G groups (columns). Each
// product is split into TF32 parts, A = Ah + Al and X = Xh + Xl (Ah, Xh the
// TF32 roundings, Al, Xl the TF32 roundings of the remainders), and
// accumulated in FP32 as Ah.Xh + Ah.Xl + Al.Xh ("3xTF32"), which keeps close
// to FP32 accuracy on the TF32 tensor pipe. A CTA gathers 64 groups into
// shared memory (split once into Xh / Xl), streams A' through shared memory
// in 32-column slices, accumulates with warp-level m16n8k8 TF32 MMAs, and
// scatters the result back.
#include <algorithm>

#include "zc_arith.cuh"
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
    static bool attr = false;
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

}  // namespace

// dev_a: [Ah (R*R) | Al (R*R)] f32 row-major, R = 2^(k+1), already TF32-rounded.
int launch_block_tc(zc_state *st, const uint32_t *qs, uint32_t k, const float *dev_a) {
    ProfScope ps(st, K_KQ, 2.0 * st->len * 4 * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * 4 * 2;
    if (st->prec != 32) return fail(ZC_ERR_UNSUPPORTED, "tensor-core blocks run on f32 states");
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
    const size_t RR = (size_t)4 << (2 * k);  // R*R with R = 2^(k+1)
    const float *ah = dev_a, *al = dev_a + RR;
    switch (k) {
        case 3: return run_tc<16>(st, p, ah, al);
        case 4: return run_tc<32>(st, p, ah, al);
        case 5: return run_tc<64>(st, p, ah, al);
        case 6: return run_tc<128>(st, p, ah, al);
        case 7: return run_tc<256>(st, p, ah, al);
        default: return fail(ZC_ERR_INVALID, "tensor-core blocks need k in 3..7");
    }
}

}  // namespace zc
