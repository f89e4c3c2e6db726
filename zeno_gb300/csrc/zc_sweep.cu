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
#include "zc_async.cuh"
#include "zc_internal.h"
#include "zc_sweep.h"

namespace zc {
namespace {

constexpr int kSweepThreads = 256;
constexpr int kSweepCtasPerSm = 3;
constexpr uint32_t kJlutHigh = 1u << (13 - 8);  // tile index values above the low byte (tiles <= 2^13)
// Global index of the first element of tile t: the tile number fills the
// non-local positions above the L low bits.
__device__ __forceinline__ uint64_t tile_base(uint64_t t, uint32_t L, const uint32_t *hpos, uint32_t H) {
    return insert_zeros(t << L, hpos, (int)H);
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

// Per-op coefficients converted once per CTA into the compute representation.
// U1: the 2x2 matrix; D1: entries 0..3 = d0r d0i d1r d1i. Double-float
// pairs for A == AR_DF, else values of T.
template <typename T, int A>
struct OpCoef {
    typename std::conditional<A == AR_DF, float2, T>::type v[8];
};

__device__ __forceinline__ bool is_1q(uint32_t kind) { return kind == MOP_U1 || kind == MOP_R1 || kind == MOP_RT; }

// The register group starting at one-qubit op o: three rotations on distinct
// bits (f64 states outside FMA mode, whose other groups are two), else up to
// kMaxGroup one-qubit ops on distinct bits. Returns its size; *rot3 tells the
// first kind.
template <typename T, int A>
__device__ __forceinline__ int group_at(const MicroOp *ops, int o, int nops, bool *rot3) {
    constexpr int kMaxGroup = sizeof(T) == 8 && A != AR_FMA ? 2 : 3;
    *rot3 = false;
    if (kMaxGroup == 2 && o + 2 < nops && ops[o].kind == MOP_RT && ops[o + 1].kind == MOP_RT &&
        ops[o + 2].kind == MOP_RT && ops[o].a != ops[o + 1].a && ops[o].a != ops[o + 2].a &&
        ops[o + 1].a != ops[o + 2].a) {
        *rot3 = true;
        return 3;
    }
    int g = 1;
    while (g < kMaxGroup && o + g < nops && is_1q(ops[o + g].kind)) {
        bool distinct = true;
        for (int h = 0; h < g; h++) distinct &= ops[o + h].a != ops[o + g].a;
        if (!distinct) break;
        g++;
    }
    return g;
}

template <typename R>
__device__ __forceinline__ uint32_t jgather(const MicroOp &op, uint32_t jo, uint32_t v) {
    uint32_t j = jo;
    for (uint32_t b = 0; b < op.k; b++)
        if (!(op.loc[b] & kOuterFlag)) j |= ((v >> op.loc[b]) & 1) << b;
    return j;
}

__device__ __forceinline__ uint32_t jouter(const MicroOp &op, uint64_t base) {
    uint32_t jo = 0;
    for (uint32_t b = 0; b < op.k; b++)
        if (op.loc[b] & kOuterFlag) jo |= (uint32_t)((base >> (op.loc[b] & ~kOuterFlag)) & 1) << b;
    return jo;
}

// Apply G consecutive one-qubit micro-ops (U1, R1 or RT; only RT when
// ROT_ONLY; ops[o..o+G), distinct tile bits) to register-held groups of 2^G
// elements: each gate updates the same pairs with the same arithmetic, in the
// same order, as one op at a time. The pair swaps of flipped RT ops commute
// with the group's other gates (other bits), so they all happen at the store:
// element e goes to the slot of e ^ flips. With FUSE_DK the table diagonal
// `dk` (the op just before the group, double-float tables) scales each
// element first, exactly as its own pass would.
template <typename T, int A, typename R, int G, bool ROT_ONLY = false, bool FUSE_DK = false>
__device__ void apply_u1_group(R *sr, R *si, const MicroOp *ops, const OpCoef<T, A> *coef, int o, uint32_t size,
                               uint32_t *bad, const MicroOp *dk = nullptr, const char *tables = nullptr,
                               uint64_t base = 0) {
    constexpr int E = 1 << G;
    uint32_t bits[G], sorted[G];
#pragma unroll
    for (int g = 0; g < G; g++) bits[g] = sorted[g] = ops[o + g].a;
#pragma unroll
    for (int i = 1; i < G; i++)
#pragma unroll
        for (int j = i; j > 0; j--)
            if (sorted[j] < sorted[j - 1]) {
                const uint32_t x = sorted[j];
                sorted[j] = sorted[j - 1];
                sorted[j - 1] = x;
            }
    uint32_t flips = 0, bad_bit = 0;
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (ops[o + g].kind == MOP_RT && ops[o + g].b) flips |= 1u << g;
        if ((1u << bits[g]) >= size) bad_bit = bits[g];
    }
    // every slot is inside the tile when the bits are (v < size / 2^G with
    // G zero bits inserted below log2(size)); a bad bit is recorded and the
    // group skipped
    if (bad_bit) {
        if (threadIdx.x == 0) *bad = bad_bit | 0x80000000u;
        return;
    }
    // flipped elements: slot(e ^ flips) = slot(e) ^ fmask
    uint32_t fmask = 0;
#pragma unroll
    for (int g = 0; g < G; g++) fmask |= ((flips >> g) & 1u) << bits[g];
    // fused diagonal: element e of the group reads table entry jb(v) ^ tp(e),
    // jb from the support bits outside the group, tp from the group's bits
    uint32_t jo = 0, tb[G];
    const float4 *dtab = nullptr;
    if constexpr (FUSE_DK) {
        jo = jouter(*dk, base);
        dtab = reinterpret_cast<const float4 *>(tables + dk->table);
#pragma unroll
        for (int g = 0; g < G; g++) {
            tb[g] = 0;
            for (uint32_t b = 0; b < dk->k; b++)
                if (dk->loc[b] == bits[g]) tb[g] = 1u << b;
        }
    }
    for (uint32_t p = threadIdx.x; p < size / E; p += blockDim.x) {
        uint32_t v = p;
#pragma unroll
        for (int g = 0; g < G; g++) v = ((v >> sorted[g]) << (sorted[g] + 1)) | (v & ((1u << sorted[g]) - 1));
        // element e of the group sits at v | (bits selected by e)
        // (recomputed at the store so the indices need no registers across
        // the arithmetic)
        auto slot = [&](uint32_t e) {
            uint32_t w = v;
#pragma unroll
            for (int g = 0; g < G; g++)
                if ((e >> g) & 1u) w ^= 1u << bits[g];
            return w;
        };
        R xr[E], xi[E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const uint32_t w = slot(e);
            xr[e] = sr[w];
            xi[e] = si[w];
        }
        if constexpr (FUSE_DK) {
            uint32_t jb = jo;
            for (uint32_t b = 0; b < dk->k; b++) {
                const uint32_t l = dk->loc[b];
                if (!(l & kOuterFlag)) jb |= ((v >> l) & 1u) << b;
            }
#pragma unroll
            for (int e = 0; e < E; e++) {
                uint32_t j = jb;
#pragma unroll
                for (int g = 0; g < G; g++)
                    if ((e >> g) & 1) j ^= tb[g];
                const float4 w = __ldg(dtab + j);
                cscale_df(make_float2(w.x, w.y), make_float2(w.z, w.w), xr[e], xi[e]);
            }
        }
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (ROT_ONLY || ops[o + g].kind == MOP_RT) {
                const R t = coef[o + g].v[0];
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (!((e >> g) & 1)) {
                        if constexpr (A == AR_DF)
                            pair_update_rot_df(t, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
                        else
                            pair_update_rot<T>(t, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
                    }
            } else if (ops[o + g].kind == MOP_R1) {
                R r[4];
#pragma unroll
                for (int i = 0; i < 4; i++) r[i] = coef[o + g].v[i];
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (!((e >> g) & 1)) {
                        if constexpr (A == AR_DF)
                            pair_update_rdf(r, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
                        else
                            pair_update_real<T>(r, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
                    }
            } else if constexpr (A == AR_DF) {
                MatDF m;
#pragma unroll
                for (int i = 0; i < 8; i++) m.v[i] = coef[o + g].v[i];
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (!((e >> g) & 1)) pair_update_df(m, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
            } else {
                Mat2<T> m;
#pragma unroll
                for (int i = 0; i < 8; i++) m.v[i] = coef[o + g].v[i];
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (!((e >> g) & 1))
                        pair_update<T, A == AR_EXACT>(m, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
            }
        }
        v ^= fmask;
#pragma unroll
        for (int e = 0; e < E; e++) {
            const uint32_t w = slot((uint32_t)e);
            sr[w] = xr[e];
            si[w] = xi[e];
        }
    }
}

// Apply the sweep's micro-ops to one tile. For A == AR_DF the tile's f64
// slots hold (hi, lo) float pairs (R = float2); otherwise R = T.
template <typename T, int A, typename R>
__device__ void apply_ops(R *sr, R *si, const MicroOp *ops, const OpCoef<T, A> *coef, int nops, uint64_t base,
                          uint32_t size, const char *tables, uint32_t *bad, uint16_t *jlut) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int o = 0; o < nops; o++) {
        const MicroOp &op = ops[o];
        if constexpr (A == AR_DF) {
            // a table diagonal right before a register group rides in its pass
            if (op.kind == MOP_DK && o + 1 < nops && is_1q(ops[o + 1].kind)) {
                bool rot3;
                const int g = group_at<T, A>(ops, o + 1, nops, &rot3);
                if (rot3)
                    apply_u1_group<T, A, R, 3, true, true>(sr, si, ops, coef, o + 1, size, bad, &op, tables, base);
                else if (g == 2)
                    apply_u1_group<T, A, R, 2, false, true>(sr, si, ops, coef, o + 1, size, bad, &op, tables, base);
                else
                    apply_u1_group<T, A, R, 1, false, true>(sr, si, ops, coef, o + 1, size, bad, &op, tables, base);
                o += g;
                __syncthreads();
                continue;
            }
        }
        if (is_1q(op.kind)) {
            // runs of up to three one-qubit ops on distinct bits share one
            // register pass (two for f64 states outside FMA mode, which would
            // spill at the 80-register cap with three, except for rotations)
            constexpr int kMaxGroup = sizeof(T) == 8 && A != AR_FMA ? 2 : 3;
            bool rot3;
            const int g = group_at<T, A>(ops, o, nops, &rot3);
            if (rot3) {
                apply_u1_group<T, A, R, 3, true>(sr, si, ops, coef, o, size, bad);
                o += 2;
                __syncthreads();
                continue;
            }
            if (kMaxGroup == 3 && g == 3) {
                apply_u1_group<T, A, R, kMaxGroup>(sr, si, ops, coef, o, size, bad);
                o += 2;
                __syncthreads();
                continue;
            }
            if (g == 2) {
                apply_u1_group<T, A, R, 2>(sr, si, ops, coef, o, size, bad);
                o += 1;
                __syncthreads();
                continue;
            }
            const uint32_t b = op.a;
            if (op.kind == MOP_RT) {
                const R t = coef[o].v[0];
                const uint32_t flip = op.b ? 1u << b : 0u;
                for (uint32_t p = tid; p < size / 2; p += nt) {
                    const uint32_t v0 = ((p >> b) << (b + 1)) | (p & ((1u << b) - 1)), v1 = v0 | (1u << b);
                    R ar = sr[v0], ai = si[v0], br = sr[v1], bi = si[v1];
                    if constexpr (A == AR_DF) pair_update_rot_df(t, ar, ai, br, bi);
                    else pair_update_rot<T>(t, ar, ai, br, bi);
                    sr[v0 ^ flip] = ar;
                    si[v0 ^ flip] = ai;
                    sr[v1 ^ flip] = br;
                    si[v1 ^ flip] = bi;
                }
                __syncthreads();
                continue;
            }
            if (op.kind == MOP_R1) {
                R r[4];
#pragma unroll
                for (int i = 0; i < 4; i++) r[i] = coef[o].v[i];
                for (uint32_t p = tid; p < size / 2; p += nt) {
                    const uint32_t v0 = ((p >> b) << (b + 1)) | (p & ((1u << b) - 1)), v1 = v0 | (1u << b);
                    if constexpr (A == AR_DF) pair_update_rdf(r, sr[v0], si[v0], sr[v1], si[v1]);
                    else pair_update_real<T>(r, sr[v0], si[v0], sr[v1], si[v1]);
                }
                __syncthreads();
                continue;
            }
            typename std::conditional<A == AR_DF, MatDF, Mat2<T>>::type m;
#pragma unroll
            for (int i = 0; i < 8; i++) m.v[i] = coef[o].v[i];
            auto upd = [&](R &ar, R &ai, R &br, R &bi) {
                if constexpr (A == AR_DF) pair_update_df(m, ar, ai, br, bi);
                else pair_update<T, A == AR_EXACT>(m, ar, ai, br, bi);
            };
            for (uint32_t p = tid; p < size / 2; p += nt) {
                const uint32_t v0 = ((p >> b) << (b + 1)) | (p & ((1u << b) - 1)), v1 = v0 | (1u << b);
                upd(sr[v0], si[v0], sr[v1], si[v1]);
            }
        } else if (op.kind == MOP_D1) {
            const bool outer = op.a & kOuterFlag;
            const bool tile_one = outer && ((base >> (op.a & ~kOuterFlag)) & 1);
            auto scl = [&](uint32_t v, R &xr, R &xi) {
                const bool one = outer ? tile_one : ((v >> op.a) & 1);
                if constexpr (A == AR_DF) cscale_df(coef[o].v[one ? 2 : 0], coef[o].v[one ? 3 : 1], xr, xi);
                else cscale<T, A == AR_EXACT>(coef[o].v[one ? 2 : 0], coef[o].v[one ? 3 : 1], xr, xi);
            };
            uint32_t v = tid;
            for (; v + 3u * nt < size; v += 4u * nt) {
                R xr[4], xi[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    xr[k] = sr[v + k * nt];
                    xi[k] = si[v + k * nt];
                }
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    scl(v + k * nt, xr[k], xi[k]);
                    sr[v + k * nt] = xr[k];
                    si[v + k * nt] = xi[k];
                }
            }
            for (; v < size; v += nt) scl(v, sr[v], si[v]);
        } else if (op.kind == MOP_DK) {
            const uint32_t jo = jouter(op, base);
            const T *dre = reinterpret_cast<const T *>(tables + op.table);
            const T *dim_ = dre + (1u << op.k);
            const float4 *dtab = reinterpret_cast<const float4 *>(tables + op.table);  // double-float entries
            // table index of element v = jo | lut[v & 255] | lut[256 + (v >> 8)]:
            // the op's local bits gathered once per op instead of per element
            for (uint32_t x = tid; x < 256 + kJlutHigh; x += nt)
                jlut[x] = (uint16_t)jgather<R>(op, 0u, x < 256 ? x : (x - 256) << 8);
            __syncthreads();
            // W: the table entry (T re, T im; or one float4 of double-float pairs)
            using W = typename std::conditional<A == AR_DF, float4, T>::type;
            auto load_w = [&](uint32_t j, W &wr, W &wi) {
                if constexpr (A == AR_DF) wr = __ldg(dtab + j);
                else {
                    wr = __ldg(dre + j);
                    wi = __ldg(dim_ + j);
                }
            };
            auto scl = [&](const W &wr, const W &wi, R &xr, R &xi) {
                if constexpr (A == AR_DF) cscale_df(make_float2(wr.x, wr.y), make_float2(wr.z, wr.w), xr, xi);
                else cscale<T, A == AR_EXACT>(wr, wi, xr, xi);
            };
            uint32_t v = tid;
            for (; v + 3u * nt < size; v += 4u * nt) {
                R xr[4], xi[4];
                W wr[4], wi[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const uint32_t vk = v + k * nt;
                    const uint32_t j = jo | jlut[vk & 255u] | jlut[256 + (vk >> 8)];
                    load_w(j, wr[k], wi[k]);
                    xr[k] = sr[vk];
                    xi[k] = si[vk];
                }
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    scl(wr[k], wi[k], xr[k], xi[k]);
                    sr[v + k * nt] = xr[k];
                    si[v + k * nt] = xi[k];
                }
            }
            for (; v < size; v += nt) {
                const uint32_t j = jo | jlut[v & 255u] | jlut[256 + (v >> 8)];
                W wr, wi;
                load_w(j, wr, wi);
                scl(wr, wi, sr[v], si[v]);
            }
        } else {
            apply_perm(sr, si, op, base, size);
        }
        __syncthreads();
    }
}

// Per-CTA state of a sweep: the current job's micro-ops, coefficients and
// row offsets, plus the tile buffer's mbarrier.
template <typename T, int A>
struct SweepSmem {
    uint64_t bar;
    MicroOp ops[kMaxMicroOps];
    OpCoef<T, A> coef[kMaxMicroOps];
    uint32_t hpos[16];     // tile bit L + j holds qubit hpos[j] (any order)
    uint32_t hsorted[16];  // the same qubits ascending (tile base)
    uint64_t row_off[1 << kMaxSweepHigh];
    int nops;
    uint32_t L, H;
    int has_arith;
    int fail;
    uint32_t fail_tile, done_tiles, bad;
    uint16_t jlut[256 + kJlutHigh];  // diagonal index tables of the current DK op
};

// All threads: make (gops, nops, L, H, hpos) the CTA's current job.
template <typename T, int A>
__device__ void load_job(SweepSmem<T, A> &c, const MicroOp *gops, int nops, uint32_t L, uint32_t H,
                         const uint32_t *hpos) {
    const int tid = threadIdx.x;
    __syncthreads();  // the previous job's tiles are done with the tables
    for (int i = tid; i < nops * (int)(sizeof(MicroOp) / 4); i += blockDim.x)
        reinterpret_cast<uint32_t *>(c.ops)[i] = reinterpret_cast<const uint32_t *>(gops)[i];
    if (tid < 16) c.hpos[tid] = tid < (int)H ? hpos[tid] : 0u;
    if (tid == 0) {
        for (uint32_t j = 0; j < H; j++) {  // insertion sort, H <= 7
            uint32_t x = hpos[j], i = j;
            for (; i > 0 && c.hsorted[i - 1] > x; i--) c.hsorted[i] = c.hsorted[i - 1];
            c.hsorted[i] = x;
        }
    }
    for (uint32_t r = tid; r < (1u << H); r += blockDim.x) {
        uint64_t o = 0;
        for (uint32_t j = 0; j < H; j++) o |= (uint64_t)((r >> j) & 1) << hpos[j];
        c.row_off[r] = o;
    }
    if (tid == 0) {
        c.nops = nops;
        c.L = L;
        c.H = H;
    }
    __syncthreads();
    if (tid < nops) {
        const MicroOp &op = c.ops[tid];
        if (op.kind == MOP_U1 || op.kind == MOP_D1 || op.kind == MOP_R1 || op.kind == MOP_RT) {
            const int cnt = op.kind == MOP_U1 ? 8 : op.kind == MOP_RT ? 1 : 4;
            for (int i = 0; i < cnt; i++) {
                if constexpr (A == AR_DF)
                    c.coef[tid].v[i] = df_from_f64(op.m[i]);
                else
                    c.coef[tid].v[i] = (T)op.m[i];
            }
        }
    }
    if (tid == 0) {
        int ar = 0;
        for (int o = 0; o < nops; o++)
            ar |= c.ops[o].kind != MOP_CX && c.ops[o].kind != MOP_SWAP;
        c.has_arith = ar;
    }
    __syncthreads();
}

// All threads: one tile of the current job — TMA row loads, micro-ops in
// shared memory, TMA row stores. Returns false if a wait ran out.
template <typename T, int A>
__device__ bool process_tile(SweepSmem<T, A> &c, T *re, T *im, uint64_t t, const char *tables, T *sre, T *sim,
                             uint32_t &phase) {
    const uint32_t size = 1u << (c.L + c.H);
    const uint32_t rows = 1u << c.H, row_elems = 1u << c.L, row_bytes = row_elems * (uint32_t)sizeof(T);
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const uint64_t base = tile_base(t, c.L, c.hsorted, c.H);
    if (warp == 0) {
        if (lane == 0) mbar_expect_tx(&c.bar, 2u * rows * row_bytes);
        __syncwarp();
        for (uint32_t r = lane; r < rows; r += 32) {
            const uint64_t gi = base | c.row_off[r];
            bulk_load(sre + (size_t)r * row_elems, re + gi, row_bytes, &c.bar);
            bulk_load(sim + (size_t)r * row_elems, im + gi, row_bytes, &c.bar);
        }
    }
    // Every thread waits; a timeout anywhere makes all threads leave together.
    if (!mbar_wait(&c.bar, phase)) {
        c.fail = 1;
        c.fail_tile = (uint32_t)t;
    }
    __syncthreads();
    if (c.fail) return false;
    phase ^= 1;
    if constexpr (A == AR_DF) {
        double *dr = reinterpret_cast<double *>(sre), *di = reinterpret_cast<double *>(sim);
        float2 *fr = reinterpret_cast<float2 *>(sre), *fi = reinterpret_cast<float2 *>(sim);
        if (c.has_arith) {
            for (uint32_t v = tid; v < size; v += blockDim.x) {
                fr[v] = df_from_f64(dr[v]);
                fi[v] = df_from_f64(di[v]);
            }
            __syncthreads();
        }
        apply_ops<T, A, float2>(fr, fi, c.ops, c.coef, c.nops, base, size, tables, &c.bad, c.jlut);
        if (c.has_arith) {
            for (uint32_t v = tid; v < size; v += blockDim.x) {
                dr[v] = df_to_f64(fr[v]);
                di[v] = df_to_f64(fi[v]);
            }
        }
    } else {
        apply_ops<T, A, T>(sre, sim, c.ops, c.coef, c.nops, base, size, tables, &c.bad, c.jlut);
    }
    fence_async_smem();
    __syncthreads();
    if (warp == 0) {
        for (uint32_t r = lane; r < rows; r += 32) {
            const uint64_t gi = base | c.row_off[r];
            bulk_store(re + gi, sre + (size_t)r * row_elems, row_bytes);
            bulk_store(im + gi, sim + (size_t)r * row_elems, row_bytes);
        }
        bulk_commit();
        bulk_wait_read_all();  // the buffer is free once the stores have read it
    }
    if (tid == 0) c.done_tiles++;
    __syncthreads();
    return true;
}

template <typename T, int A>
__device__ void sweep_init(SweepSmem<T, A> &c) {
    if (threadIdx.x == 0) {
        c.fail = 0;
        c.fail_tile = c.done_tiles = c.bad = 0;
        mbar_init(&c.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}

// Error record (the first failing CTA fills it): err[0] = 1 wait ran out /
// 2 index check; then CTA, tile, phase, raw barrier word, L, H, ops, tiles
// done, offending index.
template <typename T, int A>
__device__ void sweep_exit(SweepSmem<T, A> &c, uint32_t phase, int *err) {
    if (threadIdx.x == 0 && (c.fail || c.bad)) {
        // Give the loads still in flight a bounded chance to land before exit.
        if (c.fail) mbar_wait(&c.bar, phase);
        uint64_t raw;
        asm volatile("ld.shared.b64 %0, [%1];" : "=l"(raw) : "r"(smem_addr(&c.bar)) : "memory");
        if (atomicCAS(err, 0, c.fail ? 1 : 2) == 0) {
            err[1] = (int)blockIdx.x;
            err[2] = (int)c.fail_tile;
            err[3] = (int)phase;
            err[4] = (int)(uint32_t)raw;
            err[5] = (int)(uint32_t)(raw >> 32);
            err[6] = (int)c.L;
            err[7] = (int)c.H;
            err[8] = c.nops;
            err[9] = (int)c.done_tiles;
            err[10] = (int)c.bad;
            __threadfence();
        }
    }
    if (threadIdx.x / 32 == 0) bulk_wait_all();
}

// One state. One CTA streams tiles through a single shared-memory buffer;
// three CTAs per SM overlap one tile's TMA traffic with the others' arithmetic.
template <typename T, int A>
__global__ void __launch_bounds__(kSweepThreads, kSweepCtasPerSm)
    k_sweep(T *__restrict__ re, T *__restrict__ im, const SweepGeom g, const MicroOp *__restrict__ gops, int nops,
            const char *__restrict__ tables, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ SweepSmem<T, A> c;
    T *sre = reinterpret_cast<T *>(smem);
    T *sim = sre + (1u << (g.L + g.H));
    sweep_init(c);
    load_job(c, gops, nops, g.L, g.H, g.hpos);
    uint32_t phase = 0;
    for (uint64_t t = blockIdx.x; t < g.ntiles; t += gridDim.x)
        if (!process_tile(c, re, im, t, tables, sre, sim, phase)) break;
    sweep_exit(c, phase, err);
}

// Many states in one launch (the serving engine's packed step): the tiles
// of all jobs form one index space; a CTA switches job when its next tile
// belongs to another state.
template <typename T, int A>
__global__ void __launch_bounds__(kSweepThreads, kSweepCtasPerSm)
    k_sweep_multi(const char *__restrict__ blob, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ SweepSmem<T, A> c;
    const SweepBatch *hdr = reinterpret_cast<const SweepBatch *>(blob);
    const SweepJob *jobs = reinterpret_cast<const SweepJob *>(blob + sizeof(SweepBatch));
    const uint32_t njobs = hdr->njobs;
    const uint64_t total = hdr->total_tiles;
    sweep_init(c);
    uint32_t phase = 0;
    int cur = -1;
    // Tiles go to CTAs round-robin (concurrent tiles stay adjacent in memory
    // and big and small jobs mix evenly); the job is looked up only when a
    // tile falls outside the current one.
    uint64_t job_lo = 1, job_hi = 0;
    for (uint64_t t = blockIdx.x; t < total; t += gridDim.x) {
        if (t < job_lo || t >= job_hi) {
            uint32_t lo = 0, hi = njobs;  // last job with tile_start <= t
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) / 2;
                if (jobs[mid].tile_start <= t) lo = mid;
                else hi = mid;
            }
            const SweepJob &Jn = jobs[lo];
            load_job(c, reinterpret_cast<const MicroOp *>(blob + Jn.ops_off), (int)Jn.nops, Jn.L, Jn.H, Jn.hpos);
            cur = (int)lo;
            job_lo = Jn.tile_start;
            job_hi = Jn.tile_start + Jn.ntiles;
        }
        const SweepJob &J = jobs[cur];
        T *sre = reinterpret_cast<T *>(smem);
        T *sim = sre + (1u << (J.L + J.H));
        if (!process_tile(c, reinterpret_cast<T *>(J.re), reinterpret_cast<T *>(J.im), t - J.tile_start,
                          blob + J.tables_off, sre, sim, phase))
            break;
    }
    sweep_exit(c, phase, err);
}

template <typename T, int A>
int run_sweep(zc_state *st, const SweepGeom &g, const MicroOp *dev_ops, int nops, const char *dev_tables) {
    const size_t smem = (size_t)2 * (1u << (g.L + g.H)) * sizeof(T);
    static bool attr = false;
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_sweep<T, A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSweepSmemBytes));
        attr = true;
    }
    if (smem > kSweepSmemBytes || g.H > kMaxSweepHigh || nops > kMaxMicroOps)
        return fail(ZC_ERR_INVALID, "sweep shape exceeds the kernel's limits");
    const uint64_t blocks = std::min<uint64_t>(g.ntiles, (uint64_t)st->num_sms * kSweepCtasPerSm);
    k_sweep<T, A><<<(int)blocks, kSweepThreads, smem, st->stream>>>((T *)st->re, (T *)st->im, g, dev_ops, nops,
                                                                       dev_tables, st->d_err);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

template <typename T, int A>
int run_sweep_multi(cudaStream_t stream, int num_sms, const char *dev_blob, int *d_err) {
    static bool attr = false;
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_sweep_multi<T, A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSweepSmemBytes));
        attr = true;
    }
    k_sweep_multi<T, A><<<num_sms * kSweepCtasPerSm, kSweepThreads, kSweepSmemBytes, stream>>>(dev_blob, d_err);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

}  // namespace

int launch_sweep_multi(cudaStream_t stream, int num_sms, int prec, bool exact, const char *dev_blob, int *d_err) {
    if (prec == 64)
        return exact ? run_sweep_multi<double, AR_EXACT>(stream, num_sms, dev_blob, d_err)
                     : run_sweep_multi<double, AR_DF>(stream, num_sms, dev_blob, d_err);
    return exact ? run_sweep_multi<float, AR_EXACT>(stream, num_sms, dev_blob, d_err)
                 : run_sweep_multi<float, AR_FMA>(stream, num_sms, dev_blob, d_err);
}

int launch_sweep(zc_state *st, const SweepGeom &g, const MicroOp *dev_ops, int nops, const char *dev_tables,
                 bool exact) {
    ProfScope ps(st, K_SWEEP, 2.0 * st->len * (st->prec / 8) * 2);
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
