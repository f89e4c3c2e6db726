// Multi-op sweep kernel: one pass over HBM applies a whole run of ops.
//
// The state is cut into tiles of 2^T amplitudes: the L lowest qubits (a
// contiguous row of 2^L elements, 256 bytes) plus H chosen higher qubits
// ("local" qubits); the other n - T qubits pick the tile. A persistent CTA
// streams tiles through two shared-memory buffers: every row of a tile is
// fetched with one TMA bulk copy (cp.async.bulk, completion on an
// mbarrier), the sweep's micro-ops are applied in shared memory, and the
// rows go back with TMA bulk stores while the next tile is already in
// flight. Every micro-op uses the same arithmetic as the per-op kernels, so
// a sweep is bit-identical to launching its ops one by one.
//
// Which ops fit a sweep: unitaries whose qubits are all local; diagonals
// on any qubits (bits of non-local qubits are constant per tile); CX with a
// local target and any control; SWAP of two local qubits.
#include <algorithm>

#include "zc_arith.cuh"
#include "zc_internal.h"
#include "zc_sweep.h"

namespace zc {
namespace {

constexpr int kSweepThreads = 512;
constexpr unsigned kSpinLimit = 1u << 26;  // bounded mbarrier waits

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait on phase `parity`; returns false if the limit was reached.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_addr(bar);
    for (unsigned it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_load(void *dst_smem, const void *src_gmem, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_store(void *dst_gmem, const void *src_smem, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_gmem),
                 "r"(smem_addr(src_smem)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Global index of the first element of tile t: the tile number fills the
// non-local positions above the L low bits.
__device__ __forceinline__ uint64_t tile_base(uint64_t t, const SweepGeom &g) {
    return insert_zeros(t << g.L, g.hpos, (int)g.H);
}

__device__ __forceinline__ uint64_t row_offset(uint32_t r, const SweepGeom &g) {
    uint64_t o = 0;
    for (uint32_t j = 0; j < g.H; j++) o |= (uint64_t)((r >> j) & 1) << g.hpos[j];
    return o;
}

// Issue the bulk loads of one tile (called by all lanes of warp 0).
template <typename T>
__device__ void issue_tile_load(const T *re, const T *im, T *sre, T *sim, uint64_t base, const SweepGeom &g,
                                uint64_t *bar, int lane) {
    const uint32_t rows = 1u << g.H;
    const uint32_t row_elems = 1u << g.L;
    const uint32_t row_bytes = row_elems * sizeof(T);
    if (lane == 0) mbar_expect_tx(bar, 2u * rows * row_bytes);
    __syncwarp();
    for (uint32_t r = lane; r < rows; r += 32) {
        const uint64_t gi = base | row_offset(r, g);
        bulk_load(sre + (size_t)r * row_elems, re + gi, row_bytes, bar);
        bulk_load(sim + (size_t)r * row_elems, im + gi, row_bytes, bar);
    }
}

template <typename T>
__device__ void issue_tile_store(T *re, T *im, const T *sre, const T *sim, uint64_t base, const SweepGeom &g,
                                 int lane) {
    const uint32_t rows = 1u << g.H;
    const uint32_t row_elems = 1u << g.L;
    const uint32_t row_bytes = row_elems * sizeof(T);
    for (uint32_t r = lane; r < rows; r += 32) {
        const uint64_t gi = base | row_offset(r, g);
        bulk_store(re + gi, sre + (size_t)r * row_elems, row_bytes);
        bulk_store(im + gi, sim + (size_t)r * row_elems, row_bytes);
    }
    bulk_commit();
}

// Swap the slots v0 <-> v1 of both arrays (values of any representation).
template <typename T>
__device__ __forceinline__ void swap_slots(T *sr, T *si, uint32_t v0, uint32_t v1) {
    T x = sr[v0];
    sr[v0] = sr[v1];
    sr[v1] = x;
    x = si[v0];
    si[v0] = si[v1];
    si[v1] = x;
}

// Permutation micro-ops (CX, SWAP) move raw slots, so they serve every
// arithmetic policy and representation.
template <typename T>
__device__ void apply_perm(T *sr, T *si, const MicroOp &op, uint64_t base, uint32_t size) {
    const int tid = threadIdx.x, nt = blockDim.x;
    if (op.kind == MOP_CX) {
        const uint32_t t = op.b;
        if (op.a & kOuterFlag) {
            if (!((base >> (op.a & ~kOuterFlag)) & 1)) return;
            for (uint32_t p = tid; p < size / 2; p += nt) {
                const uint32_t v0 = ((p >> t) << (t + 1)) | (p & ((1u << t) - 1));
                swap_slots(sr, si, v0, v0 | (1u << t));
            }
        } else {
            const uint32_t c = op.a, lo = min(c, t), hi = max(c, t);
            for (uint32_t p = tid; p < size / 4; p += nt) {
                uint32_t v = ((p >> lo) << (lo + 1)) | (p & ((1u << lo) - 1));
                v = ((v >> hi) << (hi + 1)) | (v & ((1u << hi) - 1));
                const uint32_t v0 = v | (1u << c);
                swap_slots(sr, si, v0, v0 | (1u << t));
            }
        }
    } else {
        const uint32_t lo = min(op.a, op.b), hi = max(op.a, op.b);
        for (uint32_t p = tid; p < size / 4; p += nt) {
            uint32_t v = ((p >> lo) << (lo + 1)) | (p & ((1u << lo) - 1));
            v = ((v >> hi) << (hi + 1)) | (v & ((1u << hi) - 1));
            swap_slots(sr, si, v | (1u << lo), v | (1u << hi));
        }
    }
}

// Double-float micro-ops on a tile whose f64 slots hold (hi, lo) pairs.
__device__ void apply_ops_df(float2 *sr, float2 *si, const MicroOp *ops, int nops, uint64_t base,
                             const SweepGeom &g, const char *tables) {
    const uint32_t size = 1u << (g.L + g.H);
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int o = 0; o < nops; o++) {
        const MicroOp &op = ops[o];
        if (op.kind == MOP_U1) {
            const MatDF m = df_matrix(op.m);
            const uint32_t b = op.a;
            for (uint32_t p = tid; p < size / 2; p += nt) {
                const uint32_t v0 = ((p >> b) << (b + 1)) | (p & ((1u << b) - 1)), v1 = v0 | (1u << b);
                pair_update_df(m, sr[v0], si[v0], sr[v1], si[v1]);
            }
        } else if (op.kind == MOP_D1) {
            const float2 d0r = df_from_f64(op.m[0]), d0i = df_from_f64(op.m[1]);
            const float2 d1r = df_from_f64(op.m[2]), d1i = df_from_f64(op.m[3]);
            if (op.a & kOuterFlag) {
                const bool one = (base >> (op.a & ~kOuterFlag)) & 1;
                for (uint32_t v = tid; v < size; v += nt) cscale_df(one ? d1r : d0r, one ? d1i : d0i, sr[v], si[v]);
            } else {
                for (uint32_t v = tid; v < size; v += nt) {
                    const bool one = (v >> op.a) & 1;
                    cscale_df(one ? d1r : d0r, one ? d1i : d0i, sr[v], si[v]);
                }
            }
        } else if (op.kind == MOP_DK) {
            const double *dre = reinterpret_cast<const double *>(tables + op.table);
            const double *dim_ = dre + (1u << op.k);
            uint32_t jo = 0;
            for (uint32_t b = 0; b < op.k; b++)
                if (op.loc[b] & kOuterFlag) jo |= (uint32_t)((base >> (op.loc[b] & ~kOuterFlag)) & 1) << b;
            for (uint32_t v = tid; v < size; v += nt) {
                uint32_t j = jo;
                for (uint32_t b = 0; b < op.k; b++)
                    if (!(op.loc[b] & kOuterFlag)) j |= ((v >> op.loc[b]) & 1) << b;
                cscale_df(df_from_f64(__ldg(dre + j)), df_from_f64(__ldg(dim_ + j)), sr[v], si[v]);
            }
        } else {
            apply_perm(sr, si, op, base, size);
        }
        __syncthreads();
    }
}

// Apply the sweep's micro-ops to one tile held in shared memory.
template <typename T, int A>
__device__ void apply_ops(T *sr, T *si, const MicroOp *ops, int nops, uint64_t base, const SweepGeom &g,
                          const char *tables) {
    constexpr bool EXACT = A == AR_EXACT;
    const uint32_t Tb = g.L + g.H;
    const uint32_t size = 1u << Tb;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int o = 0; o < nops; o++) {
        const MicroOp &op = ops[o];
        switch (op.kind) {
            case MOP_U1: {
                Mat2<T> m;
#pragma unroll
                for (int i = 0; i < 8; i++) m.v[i] = (T)op.m[i];
                const uint32_t b = op.a;
                for (uint32_t p = tid; p < size / 2; p += nt) {
                    const uint32_t v0 = ((p >> b) << (b + 1)) | (p & ((1u << b) - 1)), v1 = v0 | (1u << b);
                    pair_update<T, EXACT>(m, sr[v0], si[v0], sr[v1], si[v1]);
                }
                break;
            }
            case MOP_D1: {
                const T d0r = (T)op.m[0], d0i = (T)op.m[1], d1r = (T)op.m[2], d1i = (T)op.m[3];
                if (op.a & kOuterFlag) {
                    const bool one = (base >> (op.a & ~kOuterFlag)) & 1;
                    const T wr = one ? d1r : d0r, wi = one ? d1i : d0i;
                    for (uint32_t v = tid; v < size; v += nt) cscale<T, EXACT>(wr, wi, sr[v], si[v]);
                } else {
                    for (uint32_t v = tid; v < size; v += nt) {
                        const bool one = (v >> op.a) & 1;
                        cscale<T, EXACT>(one ? d1r : d0r, one ? d1i : d0i, sr[v], si[v]);
                    }
                }
                break;
            }
            case MOP_DK: {
                const T *dre = reinterpret_cast<const T *>(tables + op.table);
                const T *dim_ = dre + (1u << op.k);
                uint32_t jo = 0;
                for (uint32_t b = 0; b < op.k; b++)
                    if (op.loc[b] & kOuterFlag) jo |= (uint32_t)((base >> (op.loc[b] & ~kOuterFlag)) & 1) << b;
                for (uint32_t v = tid; v < size; v += nt) {
                    uint32_t j = jo;
                    for (uint32_t b = 0; b < op.k; b++)
                        if (!(op.loc[b] & kOuterFlag)) j |= ((v >> op.loc[b]) & 1) << b;
                    cscale<T, EXACT>(__ldg(dre + j), __ldg(dim_ + j), sr[v], si[v]);
                }
                break;
            }
            case MOP_CX:
            case MOP_SWAP:
                apply_perm(sr, si, op, base, size);
                break;
            default:
                break;
        }
        __syncthreads();
    }
}

template <typename T, int A>
__global__ void __launch_bounds__(kSweepThreads, 1)
    k_sweep(T *__restrict__ re, T *__restrict__ im, const SweepGeom g, const MicroOp *__restrict__ gops, int nops,
            const char *__restrict__ tables, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ MicroOp ops[kMaxMicroOps];
    const uint32_t size = 1u << (g.L + g.H);
    T *buf_r[2], *buf_i[2];
    buf_r[0] = reinterpret_cast<T *>(smem);
    buf_i[0] = buf_r[0] + size;
    buf_r[1] = buf_i[0] + size;
    buf_i[1] = buf_r[1] + size;
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    for (int i = tid; i < nops * (int)(sizeof(MicroOp) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t *>(ops)[i] = reinterpret_cast<const uint32_t *>(gops)[i];
    bool has_arith = false;
    for (int o = 0; o < nops; o++) has_arith |= gops[o].kind == MOP_U1 || gops[o].kind == MOP_D1 || gops[o].kind == MOP_DK;
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const uint64_t first = blockIdx.x, stride = gridDim.x;
    // prefetch the first two tiles
    if (warp == 0) {
        for (int s = 0; s < 2; s++) {
            const uint64_t t = first + s * stride;
            if (t < g.ntiles) issue_tile_load(re, im, buf_r[s], buf_i[s], tile_base(t, g), g, &bars[s], lane);
        }
    }
    __shared__ int s_fail;
    if (tid == 0) s_fail = 0;
    __syncthreads();
    uint32_t phase[2] = {0, 0};
    int it = 0;
    for (uint64_t t = first; t < g.ntiles; t += stride, it++) {
        const int s = it & 1;
        // Every thread waits; a timeout anywhere makes all threads leave together.
        if (!mbar_wait(&bars[s], phase[s])) s_fail = 1;
        __syncthreads();
        if (s_fail) break;
        phase[s] ^= 1;
        const uint64_t base = tile_base(t, g);
        if constexpr (A == AR_DF) {
            // f64 slots -> (hi, lo) pairs in place, double-float ops, back to f64
            double *dr = reinterpret_cast<double *>(buf_r[s]), *di = reinterpret_cast<double *>(buf_i[s]);
            float2 *fr = reinterpret_cast<float2 *>(dr), *fi = reinterpret_cast<float2 *>(di);
            if (has_arith) {
                for (uint32_t v = tid; v < size; v += blockDim.x) {
                    fr[v] = df_from_f64(dr[v]);
                    fi[v] = df_from_f64(di[v]);
                }
                __syncthreads();
            }
            apply_ops_df(fr, fi, ops, nops, base, g, tables);
            if (has_arith) {
                for (uint32_t v = tid; v < size; v += blockDim.x) {
                    dr[v] = df_to_f64(fr[v]);
                    di[v] = df_to_f64(fi[v]);
                }
            }
        } else {
            apply_ops<T, A>(buf_r[s], buf_i[s], ops, nops, base, g, tables);
        }
        fence_async_smem();
        __syncthreads();
        if (warp == 0) {
            issue_tile_store(re, im, buf_r[s], buf_i[s], base, g, lane);
            const uint64_t tn = t + 2 * stride;
            if (tn < g.ntiles) {
                bulk_wait_read_all();  // buffer s drained before it is refilled
                issue_tile_load(re, im, buf_r[s], buf_i[s], tile_base(tn, g), g, &bars[s], lane);
            }
        }
    }
    if (s_fail) {
        // Give the loads still in flight a bounded chance to land before exit.
        if (tid == 0) {
            mbar_wait(&bars[0], phase[0]);
            mbar_wait(&bars[1], phase[1]);
            atomicExch(err, 1);
        }
    }
    if (warp == 0) bulk_wait_all();
}

template <typename T, int A>
int run_sweep(zc_state *st, const SweepGeom &g, const MicroOp *dev_ops, int nops, const char *dev_tables) {
    const size_t smem = (size_t)4 * (1u << (g.L + g.H)) * sizeof(T);
    static bool attr = false;
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_sweep<T, A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSweepSmemBytes));
        attr = true;
    }
    if (smem > kSweepSmemBytes) return fail(ZC_ERR_INVALID, "sweep tile exceeds shared memory");
    const uint64_t blocks = std::min<uint64_t>(g.ntiles, (uint64_t)st->num_sms);
    k_sweep<T, A><<<(int)blocks, kSweepThreads, smem, st->stream>>>((T *)st->re, (T *)st->im, g, dev_ops, nops,
                                                                       dev_tables, st->d_err);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

}  // namespace

int launch_sweep(zc_state *st, const SweepGeom &g, const MicroOp *dev_ops, int nops, const char *dev_tables,
                 bool exact) {
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * (st->prec / 8) * 2;
    if (st->prec == 64)
        return exact ? run_sweep<double, AR_EXACT>(st, g, dev_ops, nops, dev_tables)
                     : run_sweep<double, AR_DF>(st, g, dev_ops, nops, dev_tables);
    return exact ? run_sweep<float, AR_EXACT>(st, g, dev_ops, nops, dev_tables)
                 : run_sweep<float, AR_FMA>(st, g, dev_ops, nops, dev_tables);
}

}  // namespace zc
