// Host check of the register passes of double-float sweeps
// (zeno_gb300/csrc/zc_passes.h): random micro-op lists on one tile are
// planned into passes by plan_passes, the passes are applied the way the
// sweep kernel applies them (affine load map of the folded CX block,
// fused table diagonal indexed from the descriptor, gates in order, flipped
// stores), and the tile must equal the micro-ops applied one by one. Outer
// qubits (outside the tile) take their values from a fixed tile base.
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "zc_passes.h"

using cd = std::complex<double>;
using zc::OpHead;

namespace {

constexpr uint32_t T = 9;  // tile bits
constexpr uint32_t kSize = 1u << T;
constexpr uint32_t kOuter0 = 20, kNOuter = 6;  // outer qubits 20..25
uint64_t g_base = 0;                           // the tile's outer qubit values

struct Op {
    OpHead h;
    double m[8];
    std::vector<cd> tab;  // DK table
};

uint32_t bit_of(uint32_t slot, uint32_t x) {
    return x & zc::kOuterFlag ? (uint32_t)((g_base >> (x & ~zc::kOuterFlag)) & 1) : (slot >> x) & 1;
}

void apply_pair(std::vector<cd> &s, uint32_t a, const cd u[4]) {
    for (uint32_t i = 0; i < kSize; i++)
        if (!((i >> a) & 1)) {
            const uint32_t j = i | (1u << a);
            const cd x = s[i], y = s[j];
            s[i] = u[0] * x + u[1] * y;
            s[j] = u[2] * x + u[3] * y;
        }
}

void gate_matrix(const Op &op, cd u[4]) {
    const OpHead &h = op.h;
    if (h.kind == zc::MOP_U1) {
        for (int i = 0; i < 4; i++) u[i] = cd(op.m[2 * i], op.m[2 * i + 1]);
    } else if (h.kind == zc::MOP_R1) {
        for (int i = 0; i < 4; i++) u[i] = op.m[i];
    } else {  // RT: [[1, -t], [t, 1]], rows swapped when flipped
        const double t = op.m[0];
        const cd r[4] = {1.0, -t, t, 1.0};
        if (h.b) {
            u[0] = r[2], u[1] = r[3], u[2] = r[0], u[3] = r[1];
        } else {
            for (int i = 0; i < 4; i++) u[i] = r[i];
        }
    }
}

void apply_one(std::vector<cd> &s, const Op &op) {
    const OpHead &h = op.h;
    switch (h.kind) {
        case zc::MOP_U1:
        case zc::MOP_R1:
        case zc::MOP_RT: {
            cd u[4];
            gate_matrix(op, u);
            apply_pair(s, h.a, u);
            break;
        }
        case zc::MOP_DK:
            for (uint32_t i = 0; i < kSize; i++) {
                uint32_t j = 0;
                for (uint32_t b = 0; b < h.k; b++) j |= bit_of(i, h.loc[b]) << b;
                s[i] *= op.tab[j];
            }
            break;
        case zc::MOP_CX:
            for (uint32_t i = 0; i < kSize; i++)
                if (bit_of(i, h.a) && !((i >> h.b) & 1)) std::swap(s[i], s[i | (1u << h.b)]);
            break;
        case zc::MOP_SWAP:
            for (uint32_t i = 0; i < kSize; i++)
                if (((i >> h.a) & 1) && !((i >> h.b) & 1)) std::swap(s[i], s[(i ^ (1u << h.a)) | (1u << h.b)]);
            break;
    }
}

// One pass, as the kernel's run_pass applies it.
void apply_pass(std::vector<cd> &s, const zc::GroupInfo &q, const std::vector<Op> &ops) {
    const int G = q.G, E = 1 << G;
    uint32_t jo = 0, u0 = 0;
    for (int i = 0; i < q.nout; i++) jo |= (uint32_t)((g_base >> q.outq[i]) & 1) << q.outb[i];
    for (int t = 0; t < q.ntr; t++)
        if ((q.trc[t] & 0x80u) && ((g_base >> (q.trc[t] & 0x7fu)) & 1)) u0 ^= q.trw[t];
    const Op *dk = nullptr;
    if (q.has_dk)
        for (const Op &op : ops)
            if (op.h.kind == zc::MOP_DK && (uint32_t)op.h.table == q.tab_off) dk = &op;
    for (uint32_t p = 0; p < kSize / E; p++) {
        uint32_t v = p;
        for (int g = 0; g < G; g++) {
            const uint32_t sh = q.sorted[g];
            v = ((v >> sh) << (sh + 1)) | (v & ((1u << sh) - 1));
        }
        uint32_t lv = v ^ u0;
        for (int t = 0; t < q.ntr; t++)
            if (!(q.trc[t] & 0x80u) && ((v >> q.trc[t]) & 1)) lv ^= q.trw[t];
        std::vector<cd> x(E);
        for (int e = 0; e < E; e++) {
            uint32_t w = lv;
            for (int g = 0; g < G; g++)
                if ((e >> g) & 1) w ^= q.pm[g];
            x[e] = s[w];
        }
        if (q.has_dk) {
            uint32_t jb = jo;
            for (int i = 0; i < q.nloc; i++) jb |= ((v >> q.loc[i]) & 1u) << q.locb[i];
            for (int e = 0; e < E; e++) {
                uint32_t j = jb;
                for (int g = 0; g < G; g++)
                    if (((e >> g) & 1) && q.tb[g] != 0xff) j ^= 1u << q.tb[g];
                x[e] *= dk->tab[j];
            }
        }
        for (int g = 0; g < G; g++) {
            const Op &op = ops[q.first + g];
            cd u[4];
            if (op.h.kind == zc::MOP_RT) {  // the flip happens at the store
                const double t = op.m[0];
                u[0] = 1.0, u[1] = -t, u[2] = t, u[3] = 1.0;
            } else {
                gate_matrix(op, u);
            }
            for (int e = 0; e < E; e++)
                if (!((e >> g) & 1)) {
                    const cd a = x[e], b = x[e | (1 << g)];
                    x[e] = u[0] * a + u[1] * b;
                    x[e | (1 << g)] = u[2] * a + u[3] * b;
                }
        }
        const uint32_t vs = v ^ q.fmask;
        for (int e = 0; e < E; e++) {
            uint32_t w = vs;
            for (int g = 0; g < G; g++)
                if ((e >> g) & 1) w ^= q.gm[g];
            s[w] = x[e];
        }
    }
}

}  // namespace

int main() {
    std::mt19937_64 rng(97531);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    double worst = 0.0;
    size_t passes = 0, folded = 0, fused = 0, translations = 0;
    for (int trial = 0; trial < 3000; trial++) {
        g_base = 0;
        for (uint32_t i = 0; i < kNOuter; i++)
            if (rng() & 1) g_base |= 1ull << (kOuter0 + i);
        auto local = [&]() { return (uint32_t)(rng() % T); };
        auto outer = [&]() { return zc::kOuterFlag | (kOuter0 + (uint32_t)(rng() % kNOuter)); };
        std::vector<Op> ops;
        uint32_t tables = 0;
        auto add_gate = [&](uint32_t a) {
            Op op{};
            const int kind = (int)(rng() % 6);
            op.h.a = a;
            if (kind < 4) {
                op.h.kind = zc::MOP_RT;
                op.m[0] = U(rng);
                op.h.b = (uint32_t)(rng() & 1);
            } else if (kind < 5) {
                op.h.kind = zc::MOP_R1;
                for (int i = 0; i < 4; i++) op.m[i] = U(rng);
            } else {
                op.h.kind = zc::MOP_U1;
                for (int i = 0; i < 8; i++) op.m[i] = U(rng);
            }
            ops.push_back(op);
        };
        auto add_dk = [&]() {
            Op op{};
            op.h.kind = zc::MOP_DK;
            op.h.k = 1 + (uint32_t)(rng() % 6);
            uint64_t used = 0;
            for (uint32_t b = 0; b < op.h.k;) {
                const uint32_t x = rng() % 4 == 0 ? outer() : local();
                const uint64_t key = x & zc::kOuterFlag ? 1ull << (32 + (x & 31)) : 1ull << x;
                if (used & key) continue;
                used |= key;
                op.h.loc[b++] = x;
            }
            op.h.table = tables++;
            op.tab.resize((size_t)1 << op.h.k);
            for (auto &w : op.tab) w = std::polar(1.0, 3.0 * U(rng));
            ops.push_back(op);
        };
        auto add_cx = [&](uint32_t t) {
            Op op{};
            op.h.kind = zc::MOP_CX;
            op.h.b = t;
            do op.h.a = rng() % 3 == 0 ? outer() : local();
            while (op.h.a == t);
            ops.push_back(op);
        };
        const int len = 4 + (int)(rng() % 30);
        while ((int)ops.size() < len) {
            const int r = (int)(rng() % 10);
            if (r < 4) {  // the lowering's pattern: CX block, table diagonal, run on the targets
                uint32_t t[3];
                const int g = 1 + (int)(rng() % 3);
                for (int i = 0; i < g; i++) {
                    bool fresh;
                    do {
                        t[i] = local();
                        fresh = true;
                        for (int j = 0; j < i; j++) fresh &= t[j] != t[i];
                    } while (!fresh);
                }
                const int ncx = (int)(rng() % 4);
                for (int i = 0; i < ncx; i++) add_cx(t[rng() % g]);
                if (rng() % 3) add_dk();
                for (int i = 0; i < g; i++) add_gate(t[i]);
            } else if (r < 6) {
                add_gate(local());
            } else if (r < 7) {
                add_dk();
            } else if (r < 9) {
                add_cx(local());
            } else {
                Op op{};
                op.h.kind = zc::MOP_SWAP;
                op.h.a = local();
                do op.h.b = local();
                while (op.h.b == op.h.a);
                ops.push_back(op);
            }
        }
        std::vector<OpHead> heads;
        for (const Op &op : ops) heads.push_back(op.h);
        std::vector<cd> s0(kSize);
        for (auto &z : s0) z = cd(U(rng), U(rng));
        std::vector<cd> want = s0;
        for (const Op &op : ops) apply_one(want, op);
        // fold: the one-job kernel (the multi-job kernel plans without it);
        // max_group 2: double-float without FMA, 3: FMA arithmetic
        for (int variant = 0; variant < 4; variant++) {
            const bool fold = variant < 2;
            const int max_group = 2 + (variant & 1);
            std::vector<zc::GroupInfo> gi(ops.size());
            uint32_t bad = 0;
            int fuse_in = -1, fuse_out = -1;
            zc::plan_passes(heads.data(), (int)ops.size(), T, fold, max_group, gi.data(), &bad, &fuse_in,
                            &fuse_out);
            if (bad) {
                std::printf("FAIL trial %d variant %d: planner flagged op %u\n", trial, variant, bad & 0x7fffffffu);
                return 1;
            }
            std::vector<cd> got = s0;
            bool last_was_pass = false;
            for (size_t o = 0; o < ops.size();) {
                const zc::GroupInfo &q = gi[o];
                if (q.G) {
                    if (q.G > 3 || (q.G == 3 && max_group == 2 && !q.rot3) || q.skip < q.G ||
                        (!fold && q.ntr + (q.first - o) - (q.has_dk ? 1 : 0) != 0)) {
                        std::printf("FAIL trial %d variant %d: pass shape at op %zu\n", trial, variant, o);
                        return 1;
                    }
                    apply_pass(got, q, ops);
                    passes++;
                    folded += q.first - o - (q.has_dk ? 1 : 0);
                    fused += q.has_dk;
                    translations += q.ntr;
                    o += q.skip;
                    last_was_pass = true;
                } else {
                    apply_one(got, ops[o]);
                    o++;
                    last_was_pass = false;
                }
            }
            if (fuse_in != (gi[0].G != 0) || fuse_out != (int)last_was_pass) {
                std::printf("FAIL trial %d variant %d: fuse flags %d %d\n", trial, variant, fuse_in, fuse_out);
                return 1;
            }
            double err = 0.0, scale = 0.0;
            for (uint32_t i = 0; i < kSize; i++) {
                err = std::max(err, std::abs(got[i] - want[i]));
                scale = std::max(scale, std::abs(want[i]));
            }
            worst = std::max(worst, err / scale);
            if (err > 1e-12 * scale) {
                std::printf("FAIL trial %d variant %d: max |diff| %.3e (scale %.3e)\n", trial, variant, err, scale);
                return 1;
            }
        }
    }
    std::printf("ok worst %.3e passes %zu folded %zu fused %zu translations %zu\n", worst, passes, folded, fused,
                translations);
    return 0;
}
