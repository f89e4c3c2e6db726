// Double-float lowering of a sweep's ops (fast mode, f64 states).
//
// On GB300 the double-float arithmetic of fast f64 sweeps runs on the FP32
// pipe, and a general one-qubit gate costs four 4-term double-float dot
// products per amplitude pair. Writing U = diag(p0, p1) * R * diag(1, s1)
// with R real (r00 = |u00|, r01 = -|u01|, r10 = |u10|, r11 = |u11|) turns
// the gate into a real update (four 2-term dot products) between two
// diagonals. Diagonals commute with each other, with gates on other qubits,
// with CX on their control and, relabelled, with SWAP; through a CX on their
// target they become a diagonal that also depends on the control
// (CX D CX = D o pi, pi flipping the target bit where the control is set).
// So the lowering keeps them pending as small tables ("terms") and applies
// each term once, merged with the others, as one table-diagonal micro-op
// right before the first register run that touches its qubits. Terms still
// pending at the end of the sweep go back to the queue front as diagonal
// ops and merge into the next sweep's tables.
//
// When R is a rotation (a unitary U), R = scale * [[1, -t], [t, 1]] with
// |t| <= 1, or R = scale * [[t, -1], [1, t]] = scale * Z X [[1, t], [-t, 1]]
// (Z = diag(1, -1)): the kernel applies [[1, -t'], [t', 1]] and, for the
// second form, swaps the pair's amplitudes as it stores them; the scale and
// Z join the diagonal after it. The update is x + t*y per output, one
// double-float product.
// Rotations need few registers, so the kernel applies runs of three in one
// register pass (other runs: two); the lowering forms its runs the same way.
//
// The results agree with the unlowered sweep to the double-float rounding
// (both are within the fast mode's tolerance of the exact f64 result); the
// exact mode never lowers.
#include <algorithm>
#include <cmath>
#include <complex>

#include "zc_internal.h"

namespace zc {
namespace {

using cd = std::complex<double>;

constexpr int kTermCap = 8;   // support of a pending term
constexpr int kFlushCap = 8;  // support of one emitted table diagonal

struct Term {
    uint64_t mask;            // support: global qubits
    std::vector<cd> tab;      // index bit b <-> b-th set bit of mask (ascending)
};

uint64_t scatter(uint64_t y, uint64_t mask) {
    uint64_t g = 0;
    for (int b = 0; mask; b++) {
        const uint64_t low = mask & (~mask + 1);
        if ((y >> b) & 1) g |= low;
        mask ^= low;
    }
    return g;
}

uint64_t gather(uint64_t g, uint64_t mask) {
    uint64_t y = 0;
    for (int b = 0; mask; b++) {
        const uint64_t low = mask & (~mask + 1);
        if (g & low) y |= 1ull << b;
        mask ^= low;
    }
    return y;
}

// Term over `mask` whose value at assignment g is t(f(g)).
template <typename F>
Term remap(const Term &t, uint64_t mask, F f) {
    Term r{mask, std::vector<cd>((size_t)1 << __builtin_popcountll(mask))};
    for (uint64_t y = 0; y < r.tab.size(); y++) r.tab[y] = t.tab[gather(f(scatter(y, mask)), t.mask)];
    return r;
}

// Product of several terms over the union of their supports.
Term merge(const std::vector<Term> &ts) {
    uint64_t mask = 0;
    for (const Term &t : ts) mask |= t.mask;
    Term r{mask, std::vector<cd>((size_t)1 << __builtin_popcountll(mask), cd(1.0, 0.0))};
    for (uint64_t y = 0; y < r.tab.size(); y++) {
        const uint64_t g = scatter(y, mask);
        for (const Term &t : ts) r.tab[y] *= t.tab[gather(g, t.mask)];
    }
    return r;
}

Term one_qubit(uint32_t q, cd d0, cd d1) { return Term{1ull << q, {d0, d1}}; }

cd phase_of(cd z) { return z / std::abs(z); }

// U = diag(p0, p1) * R * diag(1, s1); false when the entries do not admit
// it to within rounding (a non-unitary matrix).
bool split_real(const double *m, double r[4], cd *s1, cd *p0, cd *p1) {
    const cd a(m[0], m[1]), b(m[2], m[3]), c(m[4], m[5]), d(m[6], m[7]);
    const cd zero(0.0, 0.0), one(1.0, 0.0);
    *p0 = a != zero ? phase_of(a) : one;
    if (b != zero) *s1 = phase_of(-b) * std::conj(*p0);
    else if (c != zero && d != zero) *s1 = phase_of(d) * std::conj(phase_of(c));
    else *s1 = one;
    *p1 = c != zero ? phase_of(c) : (d != zero ? phase_of(d) * std::conj(*s1) : one);
    r[0] = std::abs(a);
    r[1] = -std::abs(b);
    r[2] = std::abs(c);
    r[3] = std::abs(d);
    const cd got[4] = {*p0 * r[0], *p0 * r[1] * *s1, *p1 * r[2], *p1 * r[3] * *s1};
    const cd want[4] = {a, b, c, d};
    double scale = 0.0, err = 0.0;
    for (int i = 0; i < 4; i++) {
        scale = std::max(scale, std::abs(want[i]));
        err = std::max(err, std::abs(got[i] - want[i]));
    }
    return scale > 0.0 && err <= 1e-13 * scale;
}

LoweredOp diag_op(const Term &t) {
    LoweredOp o{};
    o.kind = MOP_DK;
    for (uint32_t q = 0; q < 64; q++)
        if ((t.mask >> q) & 1) o.sup.push_back(q);
    o.tab.resize(2 * t.tab.size());
    for (size_t j = 0; j < t.tab.size(); j++) {
        o.tab[2 * j] = t.tab[j].real();
        o.tab[2 * j + 1] = t.tab[j].imag();
    }
    return o;
}

// Merge `ts` into as few diagonals of at most kFlushCap qubits as a greedy
// packing gives, appending them to `out`.
void emit_terms(std::vector<Term> ts, std::vector<LoweredOp> *out) {
    while (!ts.empty()) {
        std::vector<Term> pack{ts.front()};
        uint64_t mask = ts.front().mask;
        std::vector<Term> rest;
        for (size_t i = 1; i < ts.size(); i++) {
            if (__builtin_popcountll(mask | ts[i].mask) <= kFlushCap) {
                mask |= ts[i].mask;
                pack.push_back(ts[i]);
            } else {
                rest.push_back(ts[i]);
            }
        }
        out->push_back(diag_op(merge(pack)));
        ts.swap(rest);
    }
}

// Remove the pending terms that touch `mask` and return them.
std::vector<Term> take_touching(std::vector<Term> &pending, uint64_t mask) {
    std::vector<Term> hit, keep;
    for (Term &t : pending) (t.mask & mask ? hit : keep).push_back(std::move(t));
    pending.swap(keep);
    return hit;
}

// R = scale * rotation form; false when R is not a rotation to rounding.
bool split_rot(const double *m, const double r[4], cd s1, cd p0, cd p1, int *form, double *t, double *scale) {
    const double mx = std::max(std::max(r[0], -r[1]), std::max(r[2], r[3]));
    if (std::abs(r[0] - r[3]) > 1e-15 * mx || std::abs(r[2] + r[1]) > 1e-15 * mx) return false;
    const double c = 0.5 * (r[0] + r[3]), sn = 0.5 * (r[2] - r[1]);
    double q[4];
    if (c >= sn) {
        *form = 0;
        *scale = c;
        *t = sn / c;
        q[0] = q[3] = 1.0;
        q[1] = -*t;
        q[2] = *t;
    } else {
        *form = 1;
        *scale = sn;
        *t = c / sn;
        q[0] = q[3] = *t;
        q[1] = -1.0;
        q[2] = 1.0;
    }
    const cd got[4] = {p0 * *scale * q[0], p0 * *scale * q[1] * s1, p1 * *scale * q[2], p1 * *scale * q[3] * s1};
    const cd want[4] = {cd(m[0], m[1]), cd(m[2], m[3]), cd(m[4], m[5]), cd(m[6], m[7])};
    double err = 0.0;
    for (int i = 0; i < 4; i++) err = std::max(err, std::abs(got[i] - want[i]));
    return err <= 1e-13 * mx;
}

struct Item {
    int kind;  // Q_UNITARY (one qubit), Q_DIAG, Q_CX, Q_SWAP
    uint32_t a = 0, b = 0;
    bool real = false;  // U1 written as diag * R * diag
    bool rot = false;   // ... with R = scale * rotation form
    int form = 0;
    double t = 0.0, scale = 1.0;
    double r[4] = {0, 0, 0, 0};
    cd s1, p0, p1;
    const QOp *op = nullptr;
    Term diag;  // Q_DIAG
};

bool cx_commute(const LoweredOp &x, const LoweredOp &y) {
    // CX(a, b) and CX(c, d) commute unless one's target is the other's control
    return x.b != y.a && y.b != x.a;
}

bool is_1q_op(uint32_t kind) { return kind == MOP_U1 || kind == MOP_R1 || kind == MOP_RT; }

// Size of the kernel's register group at out[i] (three rotations on distinct
// qubits, else up to run_cap one-qubit ops on distinct qubits).
size_t group_size(const std::vector<LoweredOp> &out, size_t i, int run_cap) {
    if (i + 2 < out.size() && out[i].kind == MOP_RT && out[i + 1].kind == MOP_RT && out[i + 2].kind == MOP_RT &&
        out[i].a != out[i + 1].a && out[i].a != out[i + 2].a && out[i + 1].a != out[i + 2].a)
        return 3;
    size_t g = 1;
    while ((int)g < run_cap && i + g < out.size() && is_1q_op(out[i + g].kind)) {
        bool distinct = true;
        for (size_t h = 0; h < g; h++) distinct &= out[i + h].a != out[i + g].a;
        if (!distinct) break;
        g++;
    }
    return g;
}

// The kernel takes a block of CX ops right before a register group (and its
// table diagonal) into the group's loads when every target is a group qubit,
// peeling leading CX ops that do not qualify into their own passes. Move the
// block's non-qualifying CX ops to its front where they commute with the
// qualifying ones they pass.
void arrange_cx_blocks(std::vector<LoweredOp> &out, int run_cap) {
    for (size_t i = 0; i < out.size();) {
        if (out[i].kind != MOP_CX) {
            i++;
            continue;
        }
        size_t j = i;
        while (j < out.size() && out[j].kind == MOP_CX) j++;
        const size_t g0 = j < out.size() && out[j].kind == MOP_DK ? j + 1 : j;
        if (g0 < out.size() && is_1q_op(out[g0].kind)) {
            const size_t g = group_size(out, g0, run_cap);
            auto in_group = [&](uint32_t q) {
                for (size_t h = 0; h < g; h++)
                    if (out[g0 + h].a == q) return true;
                return false;
            };
            // bubble each non-qualifying CX towards the block front
            for (size_t k = i; k < j; k++) {
                if (in_group(out[k].b)) continue;
                size_t p = k;
                while (p > i && in_group(out[p - 1].b) && cx_commute(out[p - 1], out[p])) {
                    std::swap(out[p - 1], out[p]);
                    p--;
                }
            }
        }
        i = j;
    }
}

}  // namespace

void lower_df(const std::vector<const QOp *> &seq, int run_cap, std::vector<LoweredOp> *out,
              std::vector<QOp> *carry) {
    std::vector<Item> items;
    items.reserve(seq.size());
    bool has_non_diag = false;
    for (const QOp *op : seq) {
        Item it;
        it.op = op;
        it.kind = op->kind;
        if (op->kind == Q_UNITARY) {
            const double *m = op->data.data();
            it.a = op->qs[0];
            if (m[2] == 0.0 && m[3] == 0.0 && m[4] == 0.0 && m[5] == 0.0) {
                it.kind = Q_DIAG;  // a diagonal gate is only a term
                it.diag = one_qubit(op->qs[0], cd(m[0], m[1]), cd(m[6], m[7]));
            } else {
                it.real = split_real(m, it.r, &it.s1, &it.p0, &it.p1);
                if (it.real) it.rot = split_rot(m, it.r, it.s1, it.p0, it.p1, &it.form, &it.t, &it.scale);
            }
        } else if (op->kind == Q_DIAG) {
            Term t{0, {}};
            for (uint32_t i = 0; i < op->k; i++) t.mask |= 1ull << op->qs[i];
            t.tab.resize((size_t)1 << op->k);
            for (size_t j = 0; j < t.tab.size(); j++) t.tab[j] = cd(op->data[2 * j], op->data[2 * j + 1]);
            it.diag = std::move(t);
        } else {
            it.a = op->a;
            it.b = op->b;
        }
        has_non_diag |= it.kind != Q_DIAG;
        items.push_back(std::move(it));
    }
    std::vector<Term> pending;
    for (size_t i = 0; i < items.size();) {
        Item &it = items[i];
        if (it.kind == Q_UNITARY) {
            // the register run the kernel will form: three rotations on
            // distinct qubits, else consecutive one-qubit gates on distinct
            // qubits, at most run_cap of them
            size_t j = i;
            uint64_t qmask = 0;
            const bool rot3 = i + 2 < items.size() && items[i + 1].kind == Q_UNITARY &&
                              items[i + 2].kind == Q_UNITARY && items[i].rot && items[i + 1].rot && items[i + 2].rot &&
                              items[i].a != items[i + 1].a && items[i].a != items[i + 2].a &&
                              items[i + 1].a != items[i + 2].a;
            const int cap = rot3 ? std::max(run_cap, 3) : run_cap;
            while (j < items.size() && items[j].kind == Q_UNITARY && (int)(j - i) < cap &&
                   !((qmask >> items[j].a) & 1)) {
                qmask |= 1ull << items[j].a;
                j++;
            }
            for (size_t g = i; g < j; g++)
                if (items[g].real) pending.push_back(one_qubit(items[g].a, cd(1.0, 0.0), items[g].s1));
            emit_terms(take_touching(pending, qmask), out);
            for (size_t g = i; g < j; g++) {
                LoweredOp o{};
                o.a = items[g].a;
                if (items[g].rot) {
                    o.kind = MOP_RT;
                    o.m[0] = items[g].form ? -items[g].t : items[g].t;
                    o.b = (uint32_t)items[g].form;
                } else if (items[g].real) {
                    o.kind = MOP_R1;
                    for (int k = 0; k < 4; k++) o.m[k] = items[g].r[k];
                } else {
                    o.kind = MOP_U1;
                    for (int k = 0; k < 8; k++) o.m[k] = items[g].op->data[k];
                }
                out->push_back(o);
            }
            for (size_t g = i; g < j; g++)
                if (items[g].real) {
                    // form 1: diag(p) * scale * [[t, -1], [1, t]]
                    //       = diag(-p0 * scale, p1 * scale) * X * [[1, t], [-t, 1]]
                    const double sc = items[g].rot ? items[g].scale : 1.0;
                    const double s0 = items[g].rot && items[g].form ? -sc : sc;
                    pending.push_back(one_qubit(items[g].a, items[g].p0 * s0, items[g].p1 * sc));
                }
            i = j;
            continue;
        }
        if (it.kind == Q_DIAG) {
            pending.push_back(std::move(it.diag));
        } else if (it.kind == Q_CX) {
            const uint32_t c = it.a, t = it.b;
            std::vector<Term> through = take_touching(pending, 1ull << t), flush_now;
            for (Term &d : through) {
                const uint64_t mask = d.mask | (1ull << c);
                if (__builtin_popcountll(mask) > kTermCap) {
                    flush_now.push_back(std::move(d));
                    continue;
                }
                pending.push_back(remap(d, mask, [&](uint64_t g) { return g ^ (((g >> c) & 1) << t); }));
            }
            emit_terms(std::move(flush_now), out);
            LoweredOp o{};
            o.kind = MOP_CX;
            o.a = c;
            o.b = t;
            out->push_back(o);
        } else {
            const uint32_t a = it.a, b = it.b;
            const uint64_t ab = (1ull << a) | (1ull << b);
            for (Term &d : pending) {
                if (!(d.mask & ab)) continue;
                const uint64_t ba = ((d.mask >> a) & 1) << b | ((d.mask >> b) & 1) << a;
                const uint64_t mask = (d.mask & ~ab) | ba;
                d = remap(d, mask, [&](uint64_t g) {
                    const uint64_t x = ((g >> a) ^ (g >> b)) & 1;
                    return g ^ (x << a) ^ (x << b);
                });
            }
            LoweredOp o{};
            o.kind = MOP_SWAP;
            o.a = a;
            o.b = b;
            out->push_back(o);
        }
        i++;
    }
    arrange_cx_blocks(*out, run_cap);
    if (carry && has_non_diag) {
        for (const Term &t : pending) {
            const LoweredOp d = diag_op(t);
            QOp q{};
            q.kind = Q_DIAG;
            q.k = (uint32_t)d.sup.size();
            for (uint32_t b = 0; b < q.k; b++) q.qs[b] = d.sup[b];
            q.data = d.tab;
            carry->push_back(std::move(q));
        }
    } else {
        emit_terms(std::move(pending), out);
    }
}

}  // namespace zc
