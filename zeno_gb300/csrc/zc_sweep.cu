// Multi-op sweep kernel: one pass over HBM applies a whole run of ops.
//
// The state is cut into tiles of 2^T amplitudes: the L lowest qubits (a
// contiguous row of 2^L elements, 256 bytes) plus H chosen higher qubits
// ("local" qubits); the other n - T qubits pick the tile. A persistent CTA
// streams tiles through one shared-memory buffer: every row of a tile is
// fetched with one TMA bulk copy (cp.async.bulk, completion on an
// mbarrier), the sweep's micro-ops are applied in shared memory, and the
// rows go back with TMA bulk stores; three CTAs per SM overlap one tile's
// copies with the others' arithmetic. In exact mode every micro-op uses the
// same arithmetic as the per-op kernels, so a sweep is bit-identical to
// launching its ops one by one; fast f64 sweeps run the lowered ops
// (zc_lower.cpp) in register passes of packed double-float arithmetic.
//
// Which ops fit a sweep: unitaries whose qubits are all local; diagonals
// on any qubits (bits of non-local qubits are constant per tile); CX with a
// local target and any control; SWAP of two local qubits.
#include <atomic>
#include <algorithm>

#include "zc_arith.cuh"
#include "zc_async.cuh"
#include "zc_internal.h"
#include "zc_passes.h"
#include "zc_sweep.h"

namespace zc {
namespace {

constexpr int kSweepThreads = 256;
constexpr int kSweepCtasPerSm = 3;
constexpr uint32_t kJlutHigh = 1u << (13 - 8);  // tile index values above the low byte (tiles <= 2^13)
constexpr uint32_t kJlutLen = 256 + kJlutHigh;
// Sweeps without register passes (f32 and exact f64) keep the index tables
// of their first kJobLuts table diagonals for the whole job, in the shared
// memory the pass descriptors take in double-float sweeps; further table
// diagonals build theirs per tile. A table diagonal's `b` field (in the
// CTA's copy of the micro-ops) names its job table, or kNoJobLut.
constexpr int kJobLuts = 5;
constexpr uint32_t kNoJobLut = 0xffffffffu;

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

// Swap 16-byte vectors of slots (VW consecutive elements) at v0 <-> v1.
__device__ __forceinline__ void swap_vec(void *sr, void *si, uint32_t v0, uint32_t v1) {
    uint4 *r = reinterpret_cast<uint4 *>(sr), *i = reinterpret_cast<uint4 *>(si);
    const uint4 a = r[v0], b = r[v1], c = i[v0], d = i[v1];
    r[v0] = b;
    r[v1] = a;
    i[v0] = d;
    i[v1] = c;
}

__device__ __forceinline__ uint32_t insert_zero32(uint32_t v, uint32_t b) {
    return ((v >> b) << (b + 1)) | (v & ((1u << b) - 1));
}

// Permutation micro-ops (CX, SWAP) move raw slots, so they serve every
// arithmetic policy and representation. When none of the op's bits is among
// the lowest log2(VW), the VW consecutive slots of a 16-byte vector move
// together: one vector load and store per VW elements.
template <typename T>
__device__ void apply_perm(T *sr, T *si, const OpHead &op, uint64_t base, uint32_t size) {
    const int tid = threadIdx.x, nt = blockDim.x;
    constexpr uint32_t VW = 16 / sizeof(T), VB = VW == 4 ? 2 : 1;  // elements per vector, log2
    const uint32_t nv = size / VW;                                   // vectors in the tile
    if (op.kind == MOP_CX && !(op.a & kOuterFlag) && min(op.a, op.b) >= VB) {
        const uint32_t c = op.a - VB, t = op.b - VB, lo = min(c, t), hi = max(c, t);
        for (uint32_t p = tid; p < nv / 4; p += nt) {
            const uint32_t v0 = insert_zero32(insert_zero32(p, lo), hi) | (1u << c);
            swap_vec(sr, si, v0, v0 | (1u << t));
        }
        return;
    }
    if (op.kind == MOP_CX && (op.a & kOuterFlag) && op.b >= VB) {
        if (!((base >> (op.a & ~kOuterFlag)) & 1)) return;
        const uint32_t t = op.b - VB;
        for (uint32_t p = tid; p < nv / 2; p += nt) {
            const uint32_t v0 = insert_zero32(p, t);
            swap_vec(sr, si, v0, v0 | (1u << t));
        }
        return;
    }
    if (op.kind == MOP_SWAP && min(op.a, op.b) >= VB) {
        const uint32_t lo = min(op.a, op.b) - VB, hi = max(op.a, op.b) - VB;
        for (uint32_t p = tid; p < nv / 4; p += nt) {
            const uint32_t v = insert_zero32(insert_zero32(p, lo), hi);
            swap_vec(sr, si, v | (1u << lo), v | (1u << hi));
        }
        return;
    }
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
// pairs for A == AR_DF, else values of T. Double-float RT: v[0] = t, and
// v[2..5) its packed pairs (PkReal: t hi, t lo, -t hi, each twice).
template <typename T, int A>
struct alignas(16) OpCoef {
    typename std::conditional<A == AR_DF, float2, T>::type v[8];
};

// The packed pairs of a double-float rotation's t, read where the rotation
// runs: hoisted above a group's amplitude loads, the pairs of three
// rotations (18 registers) spill at the 80-register cap.
template <typename T, int A>
__device__ __forceinline__ PkReal rot_pairs(const OpCoef<T, A> &c) {
    float4 a;
    float2 b;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w)
                 : "r"(smem_addr(&c.v[2])));
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(b.x), "=f"(b.y) : "r"(smem_addr(&c.v[4])));
    return PkReal{make_float2(a.x, a.y), make_float2(a.z, a.w), b};
}

// Double-float sweeps hold each amplitude as packed pairs: slot v of the
// re array H = (re hi, im hi), of the im array L = (re lo, im lo). The ops
// outside register passes use the scalar routines on split pairs.
__device__ __forceinline__ void hl_rot_df(float2 t, float2 &Ha, float2 &La, float2 &Hb, float2 &Lb) {
    float2 ar, ai, br, bi;
    pk_split(Ha, La, ar, ai);
    pk_split(Hb, Lb, br, bi);
    pair_update_rot_df(t, ar, ai, br, bi);
    pk_join(ar, ai, Ha, La);
    pk_join(br, bi, Hb, Lb);
}
__device__ __forceinline__ void hl_rdf(const float2 *r, float2 &Ha, float2 &La, float2 &Hb, float2 &Lb) {
    float2 ar, ai, br, bi;
    pk_split(Ha, La, ar, ai);
    pk_split(Hb, Lb, br, bi);
    pair_update_rdf(r, ar, ai, br, bi);
    pk_join(ar, ai, Ha, La);
    pk_join(br, bi, Hb, Lb);
}
__device__ __forceinline__ void hl_udf(const MatDF &m, float2 &Ha, float2 &La, float2 &Hb, float2 &Lb) {
    float2 ar, ai, br, bi;
    pk_split(Ha, La, ar, ai);
    pk_split(Hb, Lb, br, bi);
    pair_update_df(m, ar, ai, br, bi);
    pk_join(ar, ai, Ha, La);
    pk_join(br, bi, Hb, Lb);
}
// Diagonal factors leave the pairs unnormalised, as in register passes: the
// ops after them accept that, and the sweep's exit renormalises.
__device__ __forceinline__ void hl_cscale_df(float2 wr, float2 wi, float2 &H, float2 &L) {
    float2 ar, ai;
    pk_split(H, L, ar, ai);
    cscale_df_u(wr, wi, ar, ai);
    pk_join(ar, ai, H, L);
}

// The kernel's register group size: f64 states outside FMA mode spill at the
// 80-register cap with more than two general ops (rotations: three); f32
// states run groups of two as 8-byte vectors of element pairs (measured
// faster than scalar groups of three, which spill as vectors).
template <typename T, int A>
__host__ __device__ constexpr int max_group_of() {
    return sizeof(T) == 4 ? 2 : (A != AR_FMA ? 2 : 3);
}

template <typename R>
__device__ __forceinline__ uint32_t jgather(const OpHead &op, uint32_t jo, uint32_t v) {
    uint32_t j = jo;
    for (uint32_t b = 0; b < op.k; b++)
        if (!(op.loc[b] & kOuterFlag)) j |= ((v >> op.loc[b]) & 1) << b;
    return j;
}

__device__ __forceinline__ uint32_t jouter(const OpHead &op, uint64_t base) {
    uint32_t jo = 0;
    for (uint32_t b = 0; b < op.k; b++)
        if (op.loc[b] & kOuterFlag) jo |= (uint32_t)((base >> (op.loc[b] & ~kOuterFlag)) & 1) << b;
    return jo;
}

// The arithmetic of G consecutive one-qubit micro-ops (U1, R1 or RT; only RT
// when ROT_ONLY; ops[o..o+G), distinct tile bits) on a register-held group
// of 2^G elements: element e sits at the slot of the group bits selected by
// e. Each gate updates the same pairs with the same arithmetic, in the same
// order, as one op at a time.
// NE: elements held (a multiple of 2^G: several independent groups side by
// side, element e of group h at index h * 2^G + e; each gate's coefficients
// are read once for all of them).
template <typename T, int A, typename R, int G, bool ROT_ONLY, int NE = (1 << G)>
__device__ __forceinline__ void group_math(const OpHead *ops, const OpCoef<T, A> *coef, int o, R *xr, R *xi) {
    constexpr int E = NE;
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (ROT_ONLY || ops[o + g].kind == MOP_RT) {
            const R t = coef[o + g].v[0];
#pragma unroll
            for (int e = 0; e < E; e++)
                if (!((e >> g) & 1)) {
                    if constexpr (A == AR_DF)
                        hl_rot_df(t, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
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
                        hl_rdf(r, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
                    else
                        pair_update_real<T>(r, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
                }
        } else if constexpr (A == AR_DF) {
            MatDF m;
#pragma unroll
            for (int i = 0; i < 8; i++) m.v[i] = coef[o + g].v[i];
#pragma unroll
            for (int e = 0; e < E; e++)
                if (!((e >> g) & 1)) hl_udf(m, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
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
}

// The group's tile bits (bits: op order; sorted: ascending), the pattern of
// flipped RT ops and a range check. Returns false (and records the bad bit)
// when a bit lies outside the tile; `shift` counts the low bits a vector of
// consecutive elements covers (the bits are then in vector units).
template <int G>
__device__ __forceinline__ bool group_bits(const OpHead *ops, int o, uint32_t size, uint32_t shift, uint32_t *bits,
                                           uint32_t *sorted, uint32_t &fmask, uint32_t *bad) {
#pragma unroll
    for (int g = 0; g < G; g++) bits[g] = sorted[g] = ops[o + g].a - shift;
#pragma unroll
    for (int i = 1; i < G; i++)
#pragma unroll
        for (int j = i; j > 0; j--)
            if (sorted[j] < sorted[j - 1]) {
                const uint32_t x = sorted[j];
                sorted[j] = sorted[j - 1];
                sorted[j - 1] = x;
            }
    uint32_t bad_bit = 0;
    fmask = 0;
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (ops[o + g].kind == MOP_RT && ops[o + g].b) fmask |= 1u << bits[g];
        if ((1u << ops[o + g].a) >= size) bad_bit = ops[o + g].a;
    }
    // every slot is inside the tile when the bits are (v < size / 2^G with
    // G zero bits inserted below log2(size)); a bad bit is recorded and the
    // group skipped
    if (bad_bit) {
        if (threadIdx.x == 0) *bad = bad_bit | 0x80000000u;
        return false;
    }
    return true;
}

// Apply G consecutive one-qubit micro-ops to register-held groups of 2^G
// elements (group_math). The pair swaps of flipped RT ops commute with the
// group's other gates (other bits), so they all happen at the store: element
// e goes to the slot of e ^ flips.
template <typename T, int A, typename R, int G, bool ROT_ONLY = false>
__device__ void apply_u1_group(R *sr, R *si, const OpHead *ops, const OpCoef<T, A> *coef, int o, uint32_t size,
                               uint32_t *bad) {
    constexpr int E = 1 << G;
    uint32_t bits[G], sorted[G], fmask;
    if (!group_bits<G>(ops, o, size, 0u, bits, sorted, fmask, bad)) return;
    for (uint32_t p = threadIdx.x; p < size / E; p += blockDim.x) {
        uint32_t v = p;
#pragma unroll
        for (int g = 0; g < G; g++) v = ((v >> sorted[g]) << (sorted[g] + 1)) | (v & ((1u << sorted[g]) - 1));
        // element e of the group sits at v ^ (bits selected by e)
        // (recomputed at the store so the indices need no registers across
        // the arithmetic); flipped elements: slot(e ^ flips) = slot(e) ^ fmask
        auto slot = [&](uint32_t base_v, uint32_t e) {
            uint32_t w = base_v;
#pragma unroll
            for (int g = 0; g < G; g++)
                if ((e >> g) & 1u) w ^= 1u << bits[g];
            return w;
        };
        R xr[E], xi[E];
#pragma unroll
        for (int e = 0; e < E; e++) {
            const uint32_t w = slot(v, (uint32_t)e);
            xr[e] = sr[w];
            xi[e] = si[w];
        }
        group_math<T, A, R, G, ROT_ONLY>(ops, coef, o, xr, xi);
        const uint32_t vs = v ^ fmask;
#pragma unroll
        for (int e = 0; e < E; e++) {
            const uint32_t w = slot(vs, (uint32_t)e);
            sr[w] = xr[e];
            si[w] = xi[e];
        }
    }
}

// The same for 4-byte elements when no group bit is bit 0: each thread
// moves element pairs (2m, 2m + 1) as one 8-byte vector, so a group of 2^G
// vectors carries two independent element groups (the vector's two lanes)
// with half the loads, stores and index arithmetic per element.
template <typename T, int A, int G, bool ROT_ONLY = false>
__device__ void apply_u1_group_v2(float *sr, float *si, const OpHead *ops, const OpCoef<T, A> *coef, int o,
                                  uint32_t size, uint32_t *bad) {
    constexpr int E = 1 << G;
    uint32_t bits[G], sorted[G], fmask;
    if (!group_bits<G>(ops, o, size, 1u, bits, sorted, fmask, bad)) return;
    float2 *vr = reinterpret_cast<float2 *>(sr), *vi = reinterpret_cast<float2 *>(si);
    for (uint32_t p = threadIdx.x; p < size / 2 / E; p += blockDim.x) {
        uint32_t v = p;
#pragma unroll
        for (int g = 0; g < G; g++) v = ((v >> sorted[g]) << (sorted[g] + 1)) | (v & ((1u << sorted[g]) - 1));
        auto slot = [&](uint32_t base_v, uint32_t e) {
            uint32_t w = base_v;
#pragma unroll
            for (int g = 0; g < G; g++)
                if ((e >> g) & 1u) w ^= 1u << bits[g];
            return w;
        };
        float xr[2 * E], xi[2 * E];  // lane 0 (even element) at e, lane 1 at E + e
#pragma unroll
        for (int e = 0; e < E; e++) {
            const uint32_t w = slot(v, (uint32_t)e);
            const float2 a = vr[w], b = vi[w];
            xr[e] = a.x;
            xr[E + e] = a.y;
            xi[e] = b.x;
            xi[E + e] = b.y;
        }
        group_math<T, A, float, G, ROT_ONLY, 2 * E>(ops, coef, o, xr, xi);
        const uint32_t vs = v ^ fmask;
#pragma unroll
        for (int e = 0; e < E; e++) {
            const uint32_t w = slot(vs, (uint32_t)e);
            vr[w] = make_float2(xr[e], xr[E + e]);
            vi[w] = make_float2(xi[e], xi[E + e]);
        }
    }
}

// One pass (see GroupInfo) of a double-float sweep. The descriptor's fields
// are read from shared memory where they are used, which keeps the 80-register
// budget for the group's amplitudes. xr / xi hold the packed pairs H / L;
// the rotations run as f32x2 arithmetic.
// in_f64 / out_f64: the slots hold f64 on entry / must hold f64 on exit (the
// sweep's first / last pass does the tile's conversion in registers).
template <typename T, int A, int G, bool ROT_ONLY, bool HAS_DK, bool HAS_CX>
__device__ void run_pass(const GroupInfo &gi, float2 *sr, float2 *si, const OpHead *ops, const OpCoef<T, A> *coef,
                         uint32_t size, const char *tables, uint64_t base, bool in_f64, bool out_f64) {
    constexpr int E = 1 << G;
    const int o = gi.first;
    uint32_t jo = 0, u0 = 0;
    if constexpr (HAS_DK) {
        for (int i = 0; i < gi.nout; i++) jo |= (uint32_t)((base >> gi.outq[i]) & 1u) << gi.outb[i];
    }
    if constexpr (HAS_CX) {
        for (int t = 0; t < gi.ntr; t++)
            if ((gi.trc[t] & 0x80u) && ((base >> (gi.trc[t] & 0x7fu)) & 1u)) u0 ^= gi.trw[t];
    }
    for (uint32_t p = threadIdx.x; p < size / E; p += blockDim.x) {
        uint32_t v = p;
#pragma unroll
        for (int g = 0; g < G; g++) {
            const uint32_t s = gi.sorted[g];
            v = ((v >> s) << (s + 1)) | (v & ((1u << s) - 1));
        }
        float2 xr[E], xi[E];
        {
            uint32_t lv = v;
            if constexpr (HAS_CX) {
                lv ^= u0;
                for (int t = 0; t < gi.ntr; t++)
                    if (!(gi.trc[t] & 0x80u) && ((v >> gi.trc[t]) & 1u)) lv ^= gi.trw[t];
            }
#pragma unroll
            for (int e = 0; e < E; e++) {
                uint32_t w = lv;
#pragma unroll
                for (int g = 0; g < G; g++)
                    if ((e >> g) & 1) w ^= HAS_CX ? gi.pm[g] : gi.gm[g];
                if (in_f64) {
                    pk_from_f64(reinterpret_cast<const double *>(sr)[w], reinterpret_cast<const double *>(si)[w],
                                xr[e], xi[e]);
                } else {
                    xr[e] = sr[w];
                    xi[e] = si[w];
                }
            }
        }
        if constexpr (HAS_DK) {
            const float4 *dtab = reinterpret_cast<const float4 *>(tables + gi.tab_off);
            uint32_t jb = jo;
            for (int i = 0; i < gi.nloc; i++) jb |= ((v >> gi.loc[i]) & 1u) << gi.locb[i];
#pragma unroll
            for (int e = 0; e < E; e++) {
                uint32_t j = jb;
#pragma unroll
                for (int g = 0; g < G; g++)
                    if (((e >> g) & 1) && gi.tb[g] != 0xff) j ^= 1u << gi.tb[g];
                const float4 w = __ldg(dtab + j);
                float2 ar, ai;  // scalar: the packed form needs eight registers per entry
                pk_split(xr[e], xi[e], ar, ai);
                cscale_df_u(make_float2(w.x, w.y), make_float2(w.z, w.w), ar, ai);
                pk_join(ar, ai, xr[e], xi[e]);
            }
        }
        // the diagonal and the rotations chain unnormalised pairs (every
        // double-float op accepts them; |lo| grows by about an ulp of hi per
        // op, so the absolute error stays at the double-float bound);
        // renormalised only where the tile goes back to f64
#pragma unroll
        for (int g = 0; g < G; g++) {
            if (ROT_ONLY || ops[o + g].kind == MOP_RT) {
                const PkReal t = rot_pairs(coef[o + g]);
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (!((e >> g) & 1)) pk_rot_u(t, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
            } else if (ops[o + g].kind == MOP_R1) {
                float2 r[4];
#pragma unroll
                for (int i = 0; i < 4; i++) r[i] = coef[o + g].v[i];
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (!((e >> g) & 1)) hl_rdf(r, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
            } else {
                MatDF m;
#pragma unroll
                for (int i = 0; i < 8; i++) m.v[i] = coef[o + g].v[i];
#pragma unroll
                for (int e = 0; e < E; e++)
                    if (!((e >> g) & 1)) hl_udf(m, xr[e], xi[e], xr[e | (1 << g)], xi[e | (1 << g)]);
            }
        }
        const uint32_t vs = v ^ gi.fmask;
#pragma unroll
        for (int e = 0; e < E; e++) {
            uint32_t w = vs;
#pragma unroll
            for (int g = 0; g < G; g++)
                if ((e >> g) & 1) w ^= gi.gm[g];
            if (out_f64) {
                pk_to_f64(xr[e], xi[e], reinterpret_cast<double *>(sr)[w], reinterpret_cast<double *>(si)[w]);
            } else {  // the next pass accepts unnormalised pairs
                sr[w] = xr[e];
                si[w] = xi[e];
            }
        }
    }
}

template <typename T, int A, int G, bool ROT_ONLY>
__device__ void run_pass_any(const GroupInfo &gi, float2 *sr, float2 *si, const OpHead *ops,
                             const OpCoef<T, A> *coef, uint32_t size, const char *tables, uint64_t base, bool in_f64,
                             bool out_f64) {
    const bool cx = gi.ntr || gi.pm[0] != gi.gm[0] || (G > 1 && gi.pm[G - 1] != gi.gm[G - 1]) ||
                    (G > 2 && gi.pm[1] != gi.gm[1]);
    if (gi.has_dk) {
        if (cx) run_pass<T, A, G, ROT_ONLY, true, true>(gi, sr, si, ops, coef, size, tables, base, in_f64, out_f64);
        else run_pass<T, A, G, ROT_ONLY, true, false>(gi, sr, si, ops, coef, size, tables, base, in_f64, out_f64);
    } else {
        if (cx) run_pass<T, A, G, ROT_ONLY, false, true>(gi, sr, si, ops, coef, size, tables, base, in_f64, out_f64);
        else run_pass<T, A, G, ROT_ONLY, false, false>(gi, sr, si, ops, coef, size, tables, base, in_f64, out_f64);
    }
}

// gis: the job's register passes (double-float sweeps; see GroupInfo);
// fuse_in / fuse_out: its first / last pass converts the tile.
template <typename T, int A, typename R>
__device__ void apply_ops(R *sr, R *si, const OpHead *ops, const OpCoef<T, A> *coef, int nops, uint64_t base,
                          uint32_t size, const char *tables, uint32_t *bad, uint16_t *jlut, const uint16_t *job_luts,
                          const GroupInfo *gis,
                          int fuse_in = 0, int fuse_out = 0) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int o = 0; o < nops; o++) {
        const OpHead &op = ops[o];
        if constexpr (A == AR_DF) {
            const GroupInfo &gi = gis[o];
            if (gi.G) {
                const bool in_f64 = o == 0 && fuse_in, out_f64 = o + gi.skip == nops && fuse_out;
                if (gi.rot3)
                    run_pass_any<T, A, 3, true>(gi, sr, si, ops, coef, size, tables, base, in_f64, out_f64);
                else if (gi.G == 2)
                    run_pass_any<T, A, 2, false>(gi, sr, si, ops, coef, size, tables, base, in_f64, out_f64);
                else
                    run_pass_any<T, A, 1, false>(gi, sr, si, ops, coef, size, tables, base, in_f64, out_f64);
                o += gi.skip - 1;
                __syncthreads();
                continue;
            }
        }
        if (is_1q(op.kind)) {
            // runs of up to three one-qubit ops on distinct bits share one
            // register pass (two for f64 states outside FMA mode, which would
            // spill at the 80-register cap with three, except for rotations)
            constexpr int kMaxGroup = max_group_of<T, A>();
            bool rot3;
            const int g = group_at(ops, o, nops, kMaxGroup, &rot3);
            if constexpr (sizeof(R) == 4) {  // 4-byte elements: pairs of them as 8-byte vectors
                bool vec = g <= 2;
                for (int h = 0; h < g; h++) vec &= ops[o + h].a >= 1u;
                if (vec) {
                    if (g == 2) apply_u1_group_v2<T, A, 2>(sr, si, ops, coef, o, size, bad);
                    else apply_u1_group_v2<T, A, 1>(sr, si, ops, coef, o, size, bad);
                    o += g - 1;
                    __syncthreads();
                    continue;
                }
            }
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
                    if constexpr (A == AR_DF) hl_rot_df(t, ar, ai, br, bi);
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
                    if constexpr (A == AR_DF) hl_rdf(r, sr[v0], si[v0], sr[v1], si[v1]);
                    else pair_update_real<T>(r, sr[v0], si[v0], sr[v1], si[v1]);
                }
                __syncthreads();
                continue;
            }
            typename std::conditional<A == AR_DF, MatDF, Mat2<T>>::type m;
#pragma unroll
            for (int i = 0; i < 8; i++) m.v[i] = coef[o].v[i];
            auto upd = [&](R &ar, R &ai, R &br, R &bi) {
                if constexpr (A == AR_DF) hl_udf(m, ar, ai, br, bi);
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
                if constexpr (A == AR_DF) hl_cscale_df(coef[o].v[one ? 2 : 0], coef[o].v[one ? 3 : 1], xr, xi);
                else cscale<T, A == AR_EXACT>(coef[o].v[one ? 2 : 0], coef[o].v[one ? 3 : 1], xr, xi);
            };
            if constexpr (sizeof(R) == 4) {  // four consecutive elements per 16-byte vector
                float4 *vr = reinterpret_cast<float4 *>(sr), *vi = reinterpret_cast<float4 *>(si);
                for (uint32_t q = tid; q < size / 4; q += nt) {
                    const float4 a = vr[q], b = vi[q];
                    R xr[4] = {a.x, a.y, a.z, a.w}, xi[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int k = 0; k < 4; k++) scl(4 * q + k, xr[k], xi[k]);
                    vr[q] = make_float4(xr[0], xr[1], xr[2], xr[3]);
                    vi[q] = make_float4(xi[0], xi[1], xi[2], xi[3]);
                }
            } else {
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
            }
        } else if (op.kind == MOP_DK) {
            const uint32_t jo = jouter(op, base);
            // (re, im) pairs of T, or double-float (re hi, re lo, im hi, im lo)
            using P2 = typename std::conditional<sizeof(T) == 8, double2, float2>::type;
            const P2 *ptab = reinterpret_cast<const P2 *>(tables + op.table);
            const float4 *dtab = reinterpret_cast<const float4 *>(tables + op.table);
            // table index of element v = jo | lut[v & 255] | lut[256 + (v >> 8)]:
            // the op's local bits gathered once per job (or once per tile)
            // instead of per element
            const uint16_t *lut = jlut;
            if (op.b != kNoJobLut) {
                lut = job_luts + (size_t)op.b * kJlutLen;
            } else {
                for (uint32_t x = tid; x < kJlutLen; x += nt)
                    jlut[x] = (uint16_t)jgather<R>(op, 0u, x < 256 ? x : (x - 256) << 8);
                __syncthreads();
            }
            // W: the table entry (T re, T im; or one float4 of double-float pairs)
            using W = typename std::conditional<A == AR_DF, float4, T>::type;
            auto load_w = [&](uint32_t j, W &wr, W &wi) {
                if constexpr (A == AR_DF) {
                    wr = __ldg(dtab + j);
                } else {
                    const P2 w = __ldg(ptab + j);
                    wr = w.x;
                    wi = w.y;
                }
            };
            auto scl = [&](const W &wr, const W &wi, R &xr, R &xi) {
                if constexpr (A == AR_DF) hl_cscale_df(make_float2(wr.x, wr.y), make_float2(wr.z, wr.w), xr, xi);
                else cscale<T, A == AR_EXACT>(wr, wi, xr, xi);
            };
            if constexpr (sizeof(R) == 4) {  // four consecutive elements per 16-byte vector
                float4 *vr = reinterpret_cast<float4 *>(sr), *vi = reinterpret_cast<float4 *>(si);
                for (uint32_t q = tid; q < size / 4; q += nt) {
                    const uint32_t v0 = 4 * q, jh = jo | lut[256 + (v0 >> 8)];  // same high bits for all four
                    W wr[4], wi[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) load_w(jh | lut[(v0 & 255u) + k], wr[k], wi[k]);
                    const float4 a = vr[q], b = vi[q];
                    R xr[4] = {a.x, a.y, a.z, a.w}, xi[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                    for (int k = 0; k < 4; k++) scl(wr[k], wi[k], xr[k], xi[k]);
                    vr[q] = make_float4(xr[0], xr[1], xr[2], xr[3]);
                    vi[q] = make_float4(xi[0], xi[1], xi[2], xi[3]);
                }
            } else {
                uint32_t v = tid;
                for (; v + 3u * nt < size; v += 4u * nt) {
                    R xr[4], xi[4];
                    W wr[4], wi[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        const uint32_t vk = v + k * nt;
                        const uint32_t j = jo | lut[vk & 255u] | lut[256 + (vk >> 8)];
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
                    const uint32_t j = jo | lut[v & 255u] | lut[256 + (v >> 8)];
                    W wr, wi;
                    load_w(j, wr, wi);
                    scl(wr, wi, sr[v], si[v]);
                }
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
    OpHead ops[kMaxMicroOps];
    OpCoef<T, A> coef[kMaxMicroOps];
    uint32_t hpos[16];     // tile bit L + j holds qubit hpos[j] (any order)
    uint32_t hsorted[16];  // the same qubits ascending (tile base)
    int nops;
    uint32_t L, H;
    int has_arith;
    int fail;
    uint32_t fail_tile, done_tiles, bad;
    uint16_t jlut[kJlutLen];  // diagonal index tables of the current DK op
    // register passes (double-float sweeps), or the job's diagonal index tables
    typename std::conditional<A == AR_DF, GroupInfo[kMaxMicroOps], uint16_t[kJobLuts * kJlutLen]>::type gi;
    int fuse_in, fuse_out;  // the first / last pass converts the tile
};
static_assert(sizeof(uint16_t[kJobLuts * kJlutLen]) <= sizeof(GroupInfo[kMaxMicroOps]),
              "job index tables fit where the pass descriptors go");

// All threads: make (gops, nops, L, H, hpos) the CTA's current job.
template <typename T, int A>
__device__ void load_job(SweepSmem<T, A> &c, const MicroOp *gops, int nops, uint32_t L, uint32_t H,
                         const uint32_t *hpos, bool fold) {
    const int tid = threadIdx.x;
    __syncthreads();  // the previous job's tiles are done with the tables
    constexpr int kHeadWords = (int)(sizeof(OpHead) / 4), kOpWords = (int)(sizeof(MicroOp) / 4);
    for (int i = tid; i < nops * kHeadWords; i += blockDim.x)
        reinterpret_cast<uint32_t *>(c.ops)[i] =
            reinterpret_cast<const uint32_t *>(gops)[(i / kHeadWords) * kOpWords + i % kHeadWords];
    if (tid < 16) c.hpos[tid] = tid < (int)H ? hpos[tid] : 0u;
    if (tid == 0) {
        for (uint32_t j = 0; j < H; j++) {  // insertion sort, H <= 7
            uint32_t x = hpos[j], i = j;
            for (; i > 0 && c.hsorted[i - 1] > x; i--) c.hsorted[i] = c.hsorted[i - 1];
            c.hsorted[i] = x;
        }
    }
    if (tid == 0) {
        c.nops = nops;
        c.L = L;
        c.H = H;
    }
    __syncthreads();
    if (tid < nops) {
        const MicroOp &op = gops[tid];  // matrix entries from global memory
        if (op.kind == MOP_U1 || op.kind == MOP_D1 || op.kind == MOP_R1 || op.kind == MOP_RT) {
            const int cnt = op.kind == MOP_U1 ? 8 : op.kind == MOP_RT ? 1 : 4;
            for (int i = 0; i < cnt; i++) {
                if constexpr (A == AR_DF)
                    c.coef[tid].v[i] = df_from_f64(op.m[i]);
                else
                    c.coef[tid].v[i] = (T)op.m[i];
            }
            if constexpr (A == AR_DF) {
                if (op.kind == MOP_RT) {  // the rotation's packed pairs
                    const float2 t = c.coef[tid].v[0];
                    c.coef[tid].v[2] = make_float2(t.x, t.x);
                    c.coef[tid].v[3] = make_float2(t.y, t.y);
                    c.coef[tid].v[4] = make_float2(-t.x, -t.x);
                }
            }
        }
    }
    if (tid == 0) {
        int ar = 0, nlut = 0;
        for (int o = 0; o < nops; o++) {
            ar |= c.ops[o].kind != MOP_CX && c.ops[o].kind != MOP_SWAP;
            if (c.ops[o].kind == MOP_DK)
                c.ops[o].b = A != AR_DF && nlut < kJobLuts ? (uint32_t)nlut++ : kNoJobLut;
        }
        c.has_arith = ar;
        c.fuse_in = c.fuse_out = 0;
        if constexpr (A == AR_DF)
            plan_passes(c.ops, nops, L + H, fold, max_group_of<T, A>(), c.gi, &c.bad, &c.fuse_in, &c.fuse_out);
    }
    __syncthreads();
    if constexpr (A != AR_DF) {  // the job's diagonal index tables, once per job
        for (int o = 0; o < nops; o++) {
            const OpHead &op = c.ops[o];
            if (op.kind != MOP_DK || op.b == kNoJobLut) continue;
            uint16_t *lut = c.gi + (size_t)op.b * kJlutLen;
            for (uint32_t x = tid; x < kJlutLen; x += blockDim.x)
                lut[x] = (uint16_t)jgather<T>(op, 0u, x < 256 ? x : (x - 256) << 8);
        }
        __syncthreads();
    }
}

// Global offset of row r of a tile: bit j of r at qubit hpos[j].
template <typename T, int A>
__device__ __forceinline__ uint64_t row_offset(const SweepSmem<T, A> &c, uint32_t r) {
    uint64_t o = 0;
    for (uint32_t j = 0; j < c.H; j++) o |= (uint64_t)((r >> j) & 1u) << c.hpos[j];
    return o;
}

// All threads: one tile of the current job — TMA row loads, micro-ops in
// shared memory, TMA row stores. Returns false if a wait ran out.
template <typename T, int A>
__device__ bool process_tile(SweepSmem<T, A> &c, T *re, T *im, uint64_t t, const char *tables, T *sre, T *sim,
                             uint32_t &phase, uint32_t form) {
    const uint32_t size = 1u << (c.L + c.H);
    const uint32_t rows = 1u << c.H, row_elems = 1u << c.L, row_bytes = row_elems * (uint32_t)sizeof(T);
    const int tid = threadIdx.x, warp = tid / 32, lane = tid % 32;
    const uint64_t base = tile_base(t, c.L, c.hsorted, c.H);
    if (warp == 0) {
        if (lane == 0) mbar_expect_tx(&c.bar, 2u * rows * row_bytes);
        __syncwarp();
        for (uint32_t r = lane; r < rows; r += 32) {
            const uint64_t gi = base | row_offset(c, r);
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
        // The slots hold f64, or (form & kFormInDf) the normalised packed
        // pairs the previous sweep left (re slot H, im slot L); on exit f64,
        // or (form & kFormOutDf) normalised packed pairs. CX / SWAP move slots
        // whatever they hold. Each conversion reads both slots of an element
        // before it writes either.
        double *dr = reinterpret_cast<double *>(sre), *di = reinterpret_cast<double *>(sim);
        float2 *fr = reinterpret_cast<float2 *>(sre), *fi = reinterpret_cast<float2 *>(sim);
        const bool in_df = form & kFormInDf, out_df = form & kFormOutDf;
        const bool fuse_in = c.fuse_in && !in_df, fuse_out = c.fuse_out && !out_df;
        auto to_pairs = [&](uint32_t v) {
            float2 H, L;
            pk_from_f64(dr[v], di[v], H, L);
            fr[v] = H;
            fi[v] = L;
        };
        auto to_f64 = [&](uint32_t v) {
            double a, b;
            pk_to_f64(fr[v], fi[v], a, b);
            dr[v] = a;
            di[v] = b;
        };
        if (c.has_arith && !in_df && !c.fuse_in) {
            for (uint32_t v = tid; v < size; v += blockDim.x) to_pairs(v);
            __syncthreads();
        }
        apply_ops<T, A, float2>(fr, fi, c.ops, c.coef, c.nops, base, size, tables, &c.bad, c.jlut, nullptr, c.gi,
                                fuse_in,
                                fuse_out);
        if (c.has_arith && !fuse_out) {  // register passes leave pairs unnormalised
            for (uint32_t v = tid; v < size; v += blockDim.x) {
                if (out_df) {
                    float2 H = fr[v], L = fi[v];
                    pk_renorm(H, L);
                    fr[v] = H;
                    fi[v] = L;
                } else {
                    to_f64(v);
                }
            }
        } else if (!c.has_arith && in_df != out_df) {  // permutations only: change the form alone
            for (uint32_t v = tid; v < size; v += blockDim.x) {
                if (in_df) to_f64(v);
                else to_pairs(v);
            }
        }
    } else {
        apply_ops<T, A, T>(sre, sim, c.ops, c.coef, c.nops, base, size, tables, &c.bad, c.jlut, c.gi, nullptr);
    }
    fence_async_smem();
    __syncthreads();
    if (warp == 0) {
        for (uint32_t r = lane; r < rows; r += 32) {
            const uint64_t gi = base | row_offset(c, r);
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
// FORM (g.form as a compile-time constant): each hand-over of double-float
// pairs between sweeps is its own instantiation, so the tile loop carries no
// run-time branches for it (they cost registers at the 80-register cap).
template <typename T, int A, uint32_t FORM>
__global__ void __launch_bounds__(kSweepThreads, kSweepCtasPerSm)
    k_sweep(T *__restrict__ re, T *__restrict__ im, const SweepGeom g, const MicroOp *__restrict__ gops, int nops,
            const char *__restrict__ tables, int *__restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ SweepSmem<T, A> c;
    T *sre = reinterpret_cast<T *>(smem);
    T *sim = sre + (1u << (g.L + g.H));
    sweep_init(c);
    load_job(c, gops, nops, g.L, g.H, g.hpos, true);
    uint32_t phase = 0;
    for (uint64_t t = blockIdx.x; t < g.ntiles; t += gridDim.x)
        if (!process_tile(c, re, im, t, tables, sre, sim, phase, FORM)) break;
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
            // CX folding stays off here: the packed kernel's extra live state spills
            load_job(c, reinterpret_cast<const MicroOp *>(blob + Jn.ops_off), (int)Jn.nops, Jn.L, Jn.H, Jn.hpos,
                     false);
            cur = (int)lo;
            job_lo = Jn.tile_start;
            job_hi = Jn.tile_start + Jn.ntiles;
        }
        const SweepJob &J = jobs[cur];
        T *sre = reinterpret_cast<T *>(smem);
        T *sim = sre + (1u << (J.L + J.H));
        if (!process_tile(c, reinterpret_cast<T *>(J.re), reinterpret_cast<T *>(J.im), t - J.tile_start,
                          blob + J.tables_off, sre, sim, phase, 0u))
            break;
    }
    sweep_exit(c, phase, err);
}

template <typename T, int A, uint32_t FORM>
int run_sweep_form(zc_state *st, const SweepGeom &g, const MicroOp *dev_ops, int nops, const char *dev_tables) {
    const size_t smem = (size_t)2 * (1u << (g.L + g.H)) * sizeof(T);
    static std::atomic<bool> attr{false};  // set once per process; racing first calls repeat it
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_sweep<T, A, FORM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSweepSmemBytes));
        attr = true;
    }
    if (smem > kSweepSmemBytes || g.H > kMaxSweepHigh || nops > kMaxMicroOps)
        return fail(ZC_ERR_INVALID, "sweep shape exceeds the kernel's limits");
    const uint64_t blocks = std::min<uint64_t>(g.ntiles, (uint64_t)st->num_sms * kSweepCtasPerSm);
    k_sweep<T, A, FORM><<<(int)blocks, kSweepThreads, smem, st->stream>>>((T *)st->re, (T *)st->im, g, dev_ops,
                                                                             nops, dev_tables, st->d_err);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

template <typename T, int A>
int run_sweep(zc_state *st, const SweepGeom &g, const MicroOp *dev_ops, int nops, const char *dev_tables) {
    if constexpr (A == AR_DF) {
        switch (g.form) {
            case 0: return run_sweep_form<T, A, 0>(st, g, dev_ops, nops, dev_tables);
            case kFormInDf: return run_sweep_form<T, A, kFormInDf>(st, g, dev_ops, nops, dev_tables);
            case kFormOutDf: return run_sweep_form<T, A, kFormOutDf>(st, g, dev_ops, nops, dev_tables);
            default: return run_sweep_form<T, A, kFormInDf | kFormOutDf>(st, g, dev_ops, nops, dev_tables);
        }
    }
    if (g.form) return fail(ZC_ERR_INVALID, "double-float hand-over requested outside a double-float sweep");
    return run_sweep_form<T, A, 0>(st, g, dev_ops, nops, dev_tables);
}

template <typename T, int A>
int run_sweep_multi(cudaStream_t stream, int num_sms, const char *dev_blob, int *d_err) {
    static std::atomic<bool> attr{false};  // set once per process; racing first calls repeat it
    if (!attr) {
        ZC_CUDA(cudaFuncSetAttribute(k_sweep_multi<T, A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kSweepSmemBytes));
        attr = true;
    }
    k_sweep_multi<T, A><<<num_sms * kSweepCtasPerSm, kSweepThreads, kSweepSmemBytes, stream>>>(dev_blob, d_err);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

// Round a state that double-float sweeps left as packed pairs (re slot
// H = (re hi, im hi), im slot L = (re lo, im lo)) back to f64 (the last sweep
// of a flush normally does this itself; this pass serves a flush whose
// double-float sweeps are followed by another kernel).
__global__ void __launch_bounds__(256) k_df_to_f64(double *__restrict__ re, double *__restrict__ im, uint64_t len) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x) {
        const double2 a = reinterpret_cast<const double2 *>(re)[i];
        const double2 b = reinterpret_cast<const double2 *>(im)[i];
        const float4 fa = *reinterpret_cast<const float4 *>(&a), fb = *reinterpret_cast<const float4 *>(&b);
        double r0, i0, r1, i1;
        pk_to_f64(make_float2(fa.x, fa.y), make_float2(fb.x, fb.y), r0, i0);
        pk_to_f64(make_float2(fa.z, fa.w), make_float2(fb.z, fb.w), r1, i1);
        reinterpret_cast<double2 *>(re)[i] = make_double2(r0, r1);
        reinterpret_cast<double2 *>(im)[i] = make_double2(i0, i1);
    }
}

}  // namespace

int launch_df_to_f64(zc_state *st) {
    ProfScope ps(st, K_SWEEP, 2.0 * st->len * 8 * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * 8 * 2;
    const uint64_t n2 = st->len / 2;  // two elements per thread step; len >= 2^14 for sweeps
    const uint64_t blocks = std::min<uint64_t>((n2 + 255) / 256, (uint64_t)st->num_sms * 8);
    k_df_to_f64<<<(int)blocks, 256, 0, st->stream>>>((double *)st->re, (double *)st->im, n2);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

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
