// Host check of the sweep planner (zeno_gb300/csrc/zc_api.cpp plan_sweep and
// consume_plan, with the fast-mode lowering of zc_lower.cpp): random programs
// are planned sweep by sweep exactly as the library does, each sweep's encoded
// micro-ops are decoded (local tile bits back to qubits through the sweep's
// geometry) and applied to a small state, and the result must match the
// program applied directly. Links the built libzeno_cuda.so; no GPU.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "zc_internal.h"

using cd = std::complex<double>;
using zc::QOp;

static void apply_u(std::vector<cd> &s, uint32_t q, const cd m[4]) {
    for (size_t i = 0; i < s.size(); i++)
        if (!((i >> q) & 1)) {
            const size_t j = i | (size_t(1) << q);
            const cd x = s[i], y = s[j];
            s[i] = m[0] * x + m[1] * y;
            s[j] = m[2] * x + m[3] * y;
        }
}

static void apply_diag(std::vector<cd> &s, const std::vector<uint32_t> &sup, const std::vector<cd> &tab) {
    for (size_t i = 0; i < s.size(); i++) {
        size_t j = 0;
        for (size_t b = 0; b < sup.size(); b++) j |= ((i >> sup[b]) & 1) << b;
        s[i] *= tab[j];
    }
}

static void apply_cx(std::vector<cd> &s, uint32_t c, uint32_t t) {
    for (size_t i = 0; i < s.size(); i++)
        if (((i >> c) & 1) && !((i >> t) & 1)) std::swap(s[i], s[i | (size_t(1) << t)]);
}

static void apply_swap(std::vector<cd> &s, uint32_t a, uint32_t b) {
    for (size_t i = 0; i < s.size(); i++)
        if (((i >> a) & 1) && !((i >> b) & 1)) std::swap(s[i], s[(i ^ (size_t(1) << a)) | (size_t(1) << b)]);
}

static void apply_qop(std::vector<cd> &s, const QOp &op) {
    if (op.kind == zc::Q_UNITARY) {
        const cd m[4] = {{op.data[0], op.data[1]}, {op.data[2], op.data[3]}, {op.data[4], op.data[5]},
                         {op.data[6], op.data[7]}};
        apply_u(s, op.qs[0], m);
    } else if (op.kind == zc::Q_DIAG) {
        std::vector<cd> tab((size_t)1 << op.k);
        for (size_t j = 0; j < tab.size(); j++) tab[j] = cd(op.data[2 * j], op.data[2 * j + 1]);
        apply_diag(s, std::vector<uint32_t>(op.qs, op.qs + op.k), tab);
    } else if (op.kind == zc::Q_CX) {
        apply_cx(s, op.a, op.b);
    } else {
        apply_swap(s, op.a, op.b);
    }
}

// Global qubit of an encoded operand: local bit (row bits, then hpos) or
// kOuterFlag | qubit.
static uint32_t qubit_of(uint32_t x, const zc::SweepGeom &g) {
    if (x & zc::kOuterFlag) return x & ~zc::kOuterFlag;
    return x < g.L ? x : g.hpos[x - g.L];
}

static bool apply_plan(std::vector<cd> &s, const zc::SweepPlan &plan, int prec, bool ex) {
    const zc::SweepGeom &g = plan.g;
    const bool df = !ex && prec == 64;
    for (const zc::MicroOp &m : plan.mops) {
        switch (m.kind) {
            case zc::MOP_U1: {
                const cd u[4] = {{m.m[0], m.m[1]}, {m.m[2], m.m[3]}, {m.m[4], m.m[5]}, {m.m[6], m.m[7]}};
                apply_u(s, qubit_of(m.a, g), u);
                break;
            }
            case zc::MOP_R1: {
                const cd u[4] = {m.m[0], m.m[1], m.m[2], m.m[3]};
                apply_u(s, qubit_of(m.a, g), u);
                break;
            }
            case zc::MOP_RT: {  // [[1, -t], [t, 1]], then the pair's amplitudes swap when flipped
                const double t = m.m[0];
                const cd u[4] = {m.b ? t : 1.0, m.b ? 1.0 : -t, m.b ? 1.0 : t, m.b ? -t : 1.0};
                apply_u(s, qubit_of(m.a, g), u);
                break;
            }
            case zc::MOP_D1: {
                apply_diag(s, {qubit_of(m.a, g)}, {cd(m.m[0], m.m[1]), cd(m.m[2], m.m[3])});
                break;
            }
            case zc::MOP_DK: {
                std::vector<uint32_t> sup;
                for (uint32_t b = 0; b < m.k; b++) sup.push_back(qubit_of(m.loc[b], g));
                const size_t dim = (size_t)1 << m.k;
                std::vector<cd> tab(dim);
                const char *t = plan.tables.data() + m.table;
                for (size_t j = 0; j < dim; j++) {
                    if (df) {  // (re hi, re lo, im hi, im lo)
                        const float *e = (const float *)t + 4 * j;
                        tab[j] = cd((double)e[0] + (double)e[1], (double)e[2] + (double)e[3]);
                    } else if (prec == 64) {  // (re, im) pairs
                        tab[j] = cd(((const double *)t)[2 * j], ((const double *)t)[2 * j + 1]);
                    } else {
                        tab[j] = cd(((const float *)t)[2 * j], ((const float *)t)[2 * j + 1]);
                    }
                }
                apply_diag(s, sup, tab);
                break;
            }
            case zc::MOP_CX:
                apply_cx(s, qubit_of(m.a, g), qubit_of(m.b, g));
                break;
            case zc::MOP_SWAP:
                apply_swap(s, qubit_of(m.a, g), qubit_of(m.b, g));
                break;
            default:
                std::printf("FAIL: micro-op kind %u\n", m.kind);
                return false;
        }
    }
    return true;
}

int main() {
    std::mt19937_64 rng(2468);
    std::uniform_real_distribution<double> U(0.0, 2 * M_PI);
    double worst[3] = {0, 0, 0};
    size_t sweeps = 0, carried = 0;
    for (int trial = 0; trial < 300; trial++) {
        const int mode = trial % 3;  // 0 exact f64, 1 fast f64 (lowered), 2 fast f32
        const int prec = mode == 2 ? 32 : 64;
        const bool ex = mode == 0;
        // small tiles (ops on outer qubits, many sweeps), then the kernel's
        // own shape: 256-byte rows (6 bits f32, 5 bits f64) and 7 high qubits
        const bool real_shape = trial >= 240;
        const uint32_t n = real_shape ? 15 : 11;
        const uint32_t L = real_shape ? (prec == 32 ? 6u : 5u) : 3u, Hcap = real_shape ? 7u : 4u;
        std::vector<QOp> prog;
        const int len = 10 + (int)(rng() % 120);
        for (int i = 0; i < len; i++) {
            QOp op{};
            const int kind = (int)(rng() % 10);
            if (kind < 5) {
                op.kind = zc::Q_UNITARY;
                op.k = 1;
                op.qs[0] = (uint32_t)(rng() % n);
                const double th = U(rng), ph = U(rng), la = U(rng);
                cd m[4] = {std::cos(th / 2), -std::exp(cd(0, la)) * std::sin(th / 2),
                           std::exp(cd(0, ph)) * std::sin(th / 2), std::exp(cd(0, ph + la)) * std::cos(th / 2)};
                if (rng() % 6 == 0) m[1] *= cd(0, 1);  // a matrix the lowering keeps whole
                for (int k = 0; k < 4; k++) {
                    op.data.push_back(m[k].real());
                    op.data.push_back(m[k].imag());
                }
            } else if (kind < 6) {
                op.kind = zc::Q_DIAG;
                op.k = 1 + (uint32_t)(rng() % 4);
                uint32_t used = 0;
                for (uint32_t b = 0; b < op.k;) {
                    const uint32_t q = (uint32_t)(rng() % n);
                    if ((used >> q) & 1) continue;
                    used |= 1u << q;
                    b++;
                }
                for (uint32_t q = 0, b = 0; q < n; q++)
                    if ((used >> q) & 1) op.qs[b++] = q;
                for (uint32_t j = 0; j < (1u << op.k); j++) {
                    const cd w = std::exp(cd(0, U(rng)));
                    op.data.push_back(w.real());
                    op.data.push_back(w.imag());
                }
            } else {
                op.kind = kind < 9 ? zc::Q_CX : zc::Q_SWAP;
                op.a = (uint32_t)(rng() % n);
                do op.b = (uint32_t)(rng() % n);
                while (op.b == op.a);
            }
            prog.push_back(op);
        }
        std::vector<cd> s0(size_t(1) << n);
        for (auto &x : s0) x = cd(std::sin(U(rng)), std::cos(U(rng)));
        std::vector<cd> want = s0, got = s0;
        for (const QOp &op : prog) apply_qop(want, op);
        // the library's flush loop: a sweep from the queue front, or the front op alone
        std::vector<QOp> q = prog;
        int guard = 0;
        while (!q.empty()) {
            if (++guard > 100000) {
                std::printf("FAIL trial %d: planner does not make progress\n", trial);
                return 1;
            }
            zc::SweepPlan plan;
            if (zc::plan_sweep(n, prec, ex, L, Hcap, q, &plan) <= 1) {
                apply_qop(got, q.front());
                q.erase(q.begin());
                continue;
            }
            if (plan.mops.size() > (size_t)zc::kMaxMicroOps || plan.g.H > Hcap) {
                std::printf("FAIL trial %d: sweep shape %zu ops, H %u\n", trial, plan.mops.size(), plan.g.H);
                return 1;
            }
            if (!apply_plan(got, plan, prec, ex)) return 1;
            sweeps++;
            carried += plan.carry.size();
            zc::consume_plan(q, plan);
        }
        double err = 0.0;
        for (size_t i = 0; i < got.size(); i++) err = std::max(err, std::abs(got[i] - want[i]));
        worst[mode] = std::max(worst[mode], err);
        // exact mode keeps every op as given (the order of arithmetic ops
        // too); fast modes rewrite with f64 rounding; f32 tables are floats
        const double tol = mode == 2 ? 1e-5 : 1e-11;
        if (err > tol) {
            std::printf("FAIL trial %d (mode %d): max |diff| %.3e\n", trial, mode, err);
            return 1;
        }
    }
    std::printf("ok exact %.3e fast64 %.3e fast32 %.3e sweeps %zu carried %zu\n", worst[0], worst[1], worst[2],
                sweeps, carried);
    return 0;
}
