// Register passes of double-float sweeps: the micro-op head the tile loop
// reads, the pass descriptor and the planning of the passes of a job. Shared
// by the sweep kernel (zc_sweep.cu, one thread per CTA per job) and the host
// check of the pass logic (tests/passes_harness.cpp).
#pragma once
#include <stddef.h>
#include <stdint.h>

#include "zc_sweep.h"

#ifdef __CUDACC__
#define ZC_HD __host__ __device__ __forceinline__
#define ZC_HD_NOINLINE __host__ __device__ __noinline__
#else
#define ZC_HD inline
#define ZC_HD_NOINLINE inline
#endif

namespace zc {

constexpr int kMaxFoldCx = 4;  // CX ops one register group takes into its loads

// The part of a MicroOp the tile loop reads (its first 72 bytes); the matrix
// entries are read once per job, from global memory, into the coefficients.
struct OpHead {
    uint32_t kind, a, b, k;
    uint32_t loc[12];
    uint64_t table;
};
static_assert(sizeof(OpHead) == 72 && offsetof(MicroOp, table) == offsetof(OpHead, table) &&
                  offsetof(MicroOp, m) == sizeof(OpHead),
              "OpHead is the head of MicroOp");

ZC_HD bool is_1q(uint32_t kind) { return kind == MOP_U1 || kind == MOP_R1 || kind == MOP_RT; }

// The register group starting at one-qubit op o: three rotations on distinct
// bits when max_group is two (f64 states outside FMA mode), else up to
// max_group one-qubit ops on distinct bits. Returns its size; *rot3 tells the
// first kind.
ZC_HD int group_at(const OpHead *ops, int o, int nops, int max_group, bool *rot3) {
    *rot3 = false;
    if (max_group == 2 && o + 2 < nops && ops[o].kind == MOP_RT && ops[o + 1].kind == MOP_RT &&
        ops[o + 2].kind == MOP_RT && ops[o].a != ops[o + 1].a && ops[o].a != ops[o + 2].a &&
        ops[o + 1].a != ops[o + 2].a) {
        *rot3 = true;
        return 3;
    }
    int g = 1;
    while (g < max_group && o + g < nops && is_1q(ops[o + g].kind)) {
        bool distinct = true;
        for (int h = 0; h < g; h++) distinct &= ops[o + h].a != ops[o + g].a;
        if (!distinct) break;
        g++;
    }
    return g;
}

// Register passes of double-float sweeps, resolved once per job.
//
// A pass is a register group (one to three one-qubit ops on distinct tile
// bits, as group_at forms them) together with the table diagonal right
// before it and, before that, a block of CX ops whose targets are all group
// bits. The diagonal scales each element before the gates, exactly as its
// own pass would. A CX moves data only within a group whose bits hold its
// target, so the CX block becomes the load permutation: logical element y
// (group coordinates; the other bits v fixed) is read from
// pi_1(pi_2(...pi_n(y))), pi_i flipping the target where the control is
// set. Over GF(2) that is y -> M y + sum_i ctl_i(v) w_i: controls among the
// group bits make M, controls outside them (local bits of v, or outer qubits
// fixed per tile) add the translations w_i. One thread derives all of it in
// load_job; per tile a pass reads a few shared words.
struct GroupInfo {
    uint8_t G, rot3, skip, first;  // G = 0: no pass starts at this op
    uint8_t nloc, nout, ntr, has_dk;
    uint8_t sorted[3];             // group bits ascending (zero insertion)
    uint8_t tb[3];                 // table bit of each group coordinate (0xff: not in the support)
    uint8_t loc[8], locb[8];       // support bits outside the group -> table bit
    uint8_t outq[8], outb[8];      // outer support qubits -> table bit
    uint8_t trc[4];                // translation controls: local bit, or 0x80 | outer qubit
    uint16_t gm[3];                // slot pattern of group coordinate g (1 << bit)
    uint16_t pm[3];                // load pattern of coordinate g (column g of M, as slots)
    uint16_t trw[4];               // translation patterns
    uint16_t fmask;                // store pattern of the flipped coordinates
    uint32_t tab_off;
};

// One thread: walk the ops the way apply_ops will and describe each pass
// (max_group: the kernel's register group size). *fuse_in / *fuse_out: the
// job starts / ends with a pass, which then also converts the tile between
// f64 and double-float in registers.
// (Out of line on the device: one thread runs it once per job.)
ZC_HD_NOINLINE void plan_passes(const OpHead *ops, int nops, uint32_t tile_log2, bool fold, int max_group,
                                       GroupInfo *gi, uint32_t *bad, int *fuse_in, int *fuse_out) {
    for (int i = 0; i < nops; i++) gi[i].G = 0;
    *fuse_out = 0;
    int o = 0;
    while (o < nops) {
        const OpHead &op = ops[o];
        int first = -1, jdk = -1, cx0 = -1, ncx = 0;
        if (fold && op.kind == MOP_CX) {
            int j = o;
            bool ok = true;
            while (j < nops && ops[j].kind == MOP_CX && j - o < kMaxFoldCx) {
                ok &= !(ops[j].b & kOuterFlag);
                j++;
            }
            const bool dk = j < nops && ops[j].kind == MOP_DK && ops[j].k <= 8;
            const int g0 = dk ? j + 1 : j;
            if (ok && g0 < nops && is_1q(ops[g0].kind)) {
                bool rot3;
                const int g = group_at(ops, g0, nops, max_group, &rot3);
                for (int i = o; i < j; i++) {
                    bool hit = false;
                    for (int h = 0; h < g; h++) hit |= ops[g0 + h].a == ops[i].b;
                    ok &= hit;
                }
                if (ok) {
                    first = g0;
                    jdk = dk ? j : -1;
                    cx0 = o;
                    ncx = j - o;
                }
            }
        } else if (op.kind == MOP_DK && op.k <= 8 && o + 1 < nops && is_1q(ops[o + 1].kind)) {
            first = o + 1;
            jdk = o;
        } else if (is_1q(op.kind)) {
            first = o;
        }
        if (first < 0) {
            o++;
            continue;
        }
        bool rot3;
        const int G = group_at(ops, first, nops, max_group, &rot3);
        GroupInfo &q = gi[o];
        uint32_t bits[3] = {0, 0, 0};
        bool in_tile = true;
        for (int g = 0; g < G; g++) {
            bits[g] = ops[first + g].a;
            in_tile &= bits[g] < tile_log2;
        }
        if (!in_tile) {  // cannot happen for a planned sweep: recorded, ops run one by one
            *bad = 0x80000000u | (uint32_t)o;
            o++;
            continue;
        }
        q.G = (uint8_t)G;
        q.rot3 = rot3;
        q.first = (uint8_t)first;
        q.skip = (uint8_t)(first + G - o);
        q.fmask = 0;
        for (int g = 0; g < G; g++) {
            q.gm[g] = q.pm[g] = (uint16_t)(1u << bits[g]);
            if (ops[first + g].kind == MOP_RT && ops[first + g].b) q.fmask |= (uint16_t)(1u << bits[g]);
        }
        uint32_t srt[3] = {bits[0], bits[1], bits[2]};
        for (int a = 1; a < G; a++)
            for (int b = a; b > 0 && srt[b] < srt[b - 1]; b--) {
                const uint32_t x = srt[b];
                srt[b] = srt[b - 1];
                srt[b - 1] = x;
            }
        for (int g = 0; g < 3; g++) q.sorted[g] = (uint8_t)srt[g];
        q.has_dk = jdk >= 0;
        q.nloc = q.nout = 0;
        for (int g = 0; g < 3; g++) q.tb[g] = 0xff;
        if (jdk >= 0) {
            const OpHead &d = ops[jdk];
            q.tab_off = (uint32_t)d.table;
            for (uint32_t b = 0; b < d.k; b++) {
                const uint32_t l = d.loc[b];
                if (l & kOuterFlag) {
                    q.outq[q.nout] = (uint8_t)(l & ~kOuterFlag);
                    q.outb[q.nout++] = (uint8_t)b;
                    continue;
                }
                int hit = -1;
                for (int g = 0; g < G; g++)
                    if (bits[g] == l) hit = g;
                if (hit >= 0) {
                    q.tb[hit] = (uint8_t)b;
                } else {
                    q.loc[q.nloc] = (uint8_t)l;
                    q.locb[q.nloc++] = (uint8_t)b;
                }
            }
        }
        // CX block as an affine map over the group coordinates, composed
        // from the last CX (applied to y first) to the first
        q.ntr = 0;
        if (ncx > 0) {
            uint32_t col[3] = {1u, 2u, 4u}, trv[kMaxFoldCx];
            uint8_t trc[kMaxFoldCx];
            int ntr = 0;
            for (int i = ncx - 1; i >= 0; i--) {
                const OpHead &x = ops[cx0 + i];
                int tau = 0, kap = -1;
                for (int g = 0; g < G; g++) {
                    if (bits[g] == x.b) tau = g;
                    if (!(x.a & kOuterFlag) && bits[g] == x.a) kap = g;
                }
                if (kap >= 0) {  // y_tau ^= y_kap
                    for (int g = 0; g < G; g++)
                        if ((col[g] >> kap) & 1u) col[g] ^= 1u << tau;
                    for (int t = 0; t < ntr; t++)
                        if ((trv[t] >> kap) & 1u) trv[t] ^= 1u << tau;
                } else {  // y_tau ^= (control outside the group)
                    trc[ntr] = x.a & kOuterFlag ? (uint8_t)(0x80u | (x.a & ~kOuterFlag)) : (uint8_t)x.a;
                    trv[ntr++] = 1u << tau;
                }
            }
            auto pattern = [&](uint32_t y) {
                uint32_t w = 0;
                for (int g = 0; g < G; g++)
                    if ((y >> g) & 1u) w |= 1u << bits[g];
                return (uint16_t)w;
            };
            for (int g = 0; g < G; g++) q.pm[g] = pattern(col[g]);
            q.ntr = (uint8_t)ntr;
            for (int t = 0; t < ntr; t++) {
                q.trc[t] = trc[t];
                q.trw[t] = pattern(trv[t]);
            }
        }
        o += q.skip;
        *fuse_out = o == nops;
    }
    *fuse_in = nops > 0 && gi[0].G != 0;
}

}  // namespace zc
