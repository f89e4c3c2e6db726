// Host check of the double-float sweep lowering (zeno_gb300/csrc/zc_lower.cpp):
// random op sequences on a small state are applied directly and through the
// lowered ops plus the carried diagonals; the two states must agree to
// rounding. Built and run by tests/test_lowering.py with g++ (no GPU).
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "zc_internal.h"

using cd = std::complex<double>;
using zc::QOp;

static void apply_u(std::vector<cd> &s, uint32_t q, const double *m) {
    const cd a(m[0], m[1]), b(m[2], m[3]), c(m[4], m[5]), d(m[6], m[7]);
    for (size_t i = 0; i < s.size(); i++)
        if (!((i >> q) & 1)) {
            const size_t j = i | (size_t(1) << q);
            const cd x = s[i], y = s[j];
            s[i] = a * x + b * y;
            s[j] = c * x + d * y;
        }
}

static void apply_r(std::vector<cd> &s, uint32_t q, const double *r) {
    for (size_t i = 0; i < s.size(); i++)
        if (!((i >> q) & 1)) {
            const size_t j = i | (size_t(1) << q);
            const cd x = s[i], y = s[j];
            s[i] = r[0] * x + r[1] * y;
            s[j] = r[2] * x + r[3] * y;
        }
}

static void apply_diag(std::vector<cd> &s, const std::vector<uint32_t> &sup, const std::vector<double> &tab) {
    for (size_t i = 0; i < s.size(); i++) {
        size_t j = 0;
        for (size_t b = 0; b < sup.size(); b++) j |= ((i >> sup[b]) & 1) << b;
        s[i] *= cd(tab[2 * j], tab[2 * j + 1]);
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
    if (op.kind == zc::Q_UNITARY) apply_u(s, op.qs[0], op.data.data());
    else if (op.kind == zc::Q_DIAG) apply_diag(s, std::vector<uint32_t>(op.qs, op.qs + op.k), op.data);
    else if (op.kind == zc::Q_CX) apply_cx(s, op.a, op.b);
    else apply_swap(s, op.a, op.b);
}

static void apply_lowered(std::vector<cd> &s, const zc::LoweredOp &o) {
    switch (o.kind) {
        case zc::MOP_U1: apply_u(s, o.a, o.m); break;
        case zc::MOP_R1: apply_r(s, o.a, o.m); break;
        case zc::MOP_RT: {  // [[1, -t], [t, 1]], then the pair's amplitudes swap when flipped
            const double t = o.m[0];
            const double r[4] = {o.b ? t : 1.0, o.b ? 1.0 : -t, o.b ? 1.0 : t, o.b ? -t : 1.0};
            apply_r(s, o.a, r);
            break;
        }
        case zc::MOP_DK: apply_diag(s, o.sup, o.tab); break;
        case zc::MOP_CX: apply_cx(s, o.a, o.b); break;
        case zc::MOP_SWAP: apply_swap(s, o.a, o.b); break;
        default: std::printf("bad kind %u\n", o.kind); std::exit(2);
    }
}

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 2 * M_PI);
    const uint32_t n = 7;
    double worst = 0.0;
    size_t total_r1 = 0, total_rt = 0, total_u1 = 0, total_dk = 0, total_carry = 0, total_gates = 0;
    for (int trial = 0; trial < 400; trial++) {
        std::vector<QOp> prog;
        const int len = 1 + (int)(rng() % 40);
        for (int i = 0; i < len; i++) {
            QOp op{};
            const int kind = (int)(rng() % 10);
            if (kind < 5) {  // u3, or a special one-qubit matrix
                op.kind = zc::Q_UNITARY;
                op.k = 1;
                op.qs[0] = (uint32_t)(rng() % n);
                const double th = U(rng), ph = U(rng), la = U(rng);
                cd m[4] = {std::cos(th / 2), -std::exp(cd(0, la)) * std::sin(th / 2),
                           std::exp(cd(0, ph)) * std::sin(th / 2), std::exp(cd(0, ph + la)) * std::cos(th / 2)};
                const int sp = (int)(rng() % 8);
                if (sp == 0) {  // X
                    m[0] = m[3] = 0;
                    m[1] = m[2] = 1;
                } else if (sp == 1) {  // S (diagonal)
                    m[0] = 1;
                    m[1] = m[2] = 0;
                    m[3] = cd(0, 1);
                } else if (sp == 2) {  // H
                    m[0] = m[1] = m[2] = 1 / std::sqrt(2.0);
                    m[3] = -1 / std::sqrt(2.0);
                } else if (sp == 3) {  // phases no diagonal * real * diagonal can give: kept whole
                    m[1] *= cd(0, 1);
                } else if (sp == 4) {  // not unitary, but the split holds entry by entry
                    m[1] *= 1.5;
                }
                for (int k = 0; k < 4; k++) {
                    op.data.push_back(m[k].real());
                    op.data.push_back(m[k].imag());
                }
                total_gates++;
            } else if (kind < 6) {
                op.kind = zc::Q_DIAG;
                op.k = 1 + (uint32_t)(rng() % 3);
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
        std::vector<const QOp *> seq;
        for (const QOp &op : prog) seq.push_back(&op);
        std::vector<zc::LoweredOp> low;
        std::vector<QOp> carry;
        const bool use_carry = trial % 2 == 0;
        zc::lower_df(seq, 2 + trial % 2, &low, use_carry ? &carry : nullptr);
        for (const auto &o : low) {
            apply_lowered(got, o);
            total_r1 += o.kind == zc::MOP_R1;
            total_rt += o.kind == zc::MOP_RT;
            total_u1 += o.kind == zc::MOP_U1;
            total_dk += o.kind == zc::MOP_DK;
            if (o.kind == zc::MOP_DK && (o.sup.empty() || o.sup.size() > 12)) {
                std::printf("FAIL trial %d: table support %zu\n", trial, o.sup.size());
                return 1;
            }
        }
        for (const QOp &op : carry) {
            if (op.kind != zc::Q_DIAG || op.k < 1 || op.k > 12) {
                std::printf("FAIL trial %d: bad carried op\n", trial);
                return 1;
            }
            apply_qop(got, op);
        }
        total_carry += carry.size();
        double err = 0.0;
        for (size_t i = 0; i < got.size(); i++) err = std::max(err, std::abs(got[i] - want[i]));
        worst = std::max(worst, err);
        if (err > 1e-12) {
            std::printf("FAIL trial %d: max |diff| %.3e (len %d)\n", trial, err, len);
            return 1;
        }
    }
    std::printf("ok worst %.3e gates %zu r1 %zu rt %zu u1 %zu dk %zu carried %zu\n", worst, total_gates, total_r1,
                total_rt, total_u1, total_dk, total_carry);
    return 0;
}
