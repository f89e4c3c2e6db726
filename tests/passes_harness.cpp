// Host check of the register passes of double-float sweeps
// (zeno_gb300/csrc/zc_passes.h): random micro-op lists on one tile are
// planned into passes by plan_passes, the passes are applied the way the
// sweep kernel applies them (affine load map of the folded CX block,
// fused table diagonal indexed from the descriptor, gates in order, flipped
// stores), and the tile must equal the micro-ops applied one by one. Outer
// qubits (outside the tile) take their values from a fixed tile base.
#include "tile_ref.h"

using namespace tile_ref;

namespace {

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
    for (uint32_t p = 0; p < g_size / E; p++) {
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
    Gen gen(97531);
    double worst = 0.0;
    size_t passes = 0, folded = 0, fused = 0, translations = 0;
    for (int trial = 0; trial < 3400; trial++) {
        // 2^9-element tiles, then the double-float kernel's own 2^12
        set_tile_bits(trial < 3000 ? 9 : 12);
        gen.new_base();
        const std::vector<Op> ops = gen.list(30);
        std::vector<OpHead> heads;
        for (const Op &op : ops) heads.push_back(op.h);
        std::vector<cd> s0(g_size);
        for (auto &z : s0) z = cd(gen.U(gen.rng), gen.U(gen.rng));
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
            zc::plan_passes(heads.data(), (int)ops.size(), g_tile_bits, fold, max_group, gi.data(), &bad, &fuse_in,
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
            const double d = rel_diff(got, want);
            worst = std::max(worst, d);
            if (d > 1e-12) {
                std::printf("FAIL trial %d variant %d: max |diff| %.3e relative\n", trial, variant, d);
                return 1;
            }
        }
    }
    std::printf("ok worst %.3e passes %zu folded %zu fused %zu translations %zu\n", worst, passes, folded, fused,
                translations);
    return 0;
}
