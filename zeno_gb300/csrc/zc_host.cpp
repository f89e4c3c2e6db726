// Host pipeline above the backend: native gate matrices, the fusion
// compiler and the executor (run_sampled / run_per_shot with trajectory
// noise). Same passes and the same floating-point evaluation order as the
// reference, so fused matrices are bit-identical to zeno's for a given
// libm; extended for the GPU with 7-qubit dense fusion and SWAP kept as a
// zero-arithmetic permutation op.
//
//   gates       src/gates.rs:30-188
//   compiler    src/compiler.rs:118-626
//   executor    src/exec.rs:347-619
//   noise       src/noise.rs:91-192
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include "zc_internal.h"
#include "zc_rng.h"
#include "zc_traj.h"

namespace zc {
namespace {

// Complex value with num-complex 0.4 arithmetic (no library complex: its
// multiply may special-case or contract).
struct Cx {
    double re = 0.0, im = 0.0;
};
inline Cx mk(double r, double i) { return Cx{r, i}; }
inline Cx operator*(Cx a, Cx b) { return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
inline Cx operator+(Cx a, Cx b) { return mk(a.re + b.re, a.im + b.im); }
inline Cx scale(Cx a, double s) { return mk(a.re * s, a.im * s); }
inline Cx neg(Cx a) { return mk(-a.re, -a.im); }
inline Cx expi(double t) { return mk(cos(t), sin(t)); }
inline bool is_zero(Cx a) { return a.re == 0.0 && a.im == 0.0; }

using Mat = std::vector<Cx>;

// ------------------------------------------------------------------ gates

struct GateDef {
    const char *name;
    int arity, nparams;
};

const GateDef kGates[] = {
    {"id", 1, 0},  {"u0", 1, 0},   {"x", 1, 0},    {"y", 1, 0},   {"z", 1, 0},   {"h", 1, 0},   {"s", 1, 0},
    {"sdg", 1, 0}, {"t", 1, 0},    {"tdg", 1, 0},  {"sx", 1, 0},  {"sxdg", 1, 0}, {"rx", 1, 1}, {"ry", 1, 1},
    {"rz", 1, 1},  {"u1", 1, 1},   {"p", 1, 1},    {"u2", 1, 2},  {"u3", 1, 3},  {"u", 1, 3},   {"cx", 2, 0},
    {"cy", 2, 0},  {"cz", 2, 0},   {"ch", 2, 0},   {"swap", 2, 0}, {"cp", 2, 1}, {"cu1", 2, 1}, {"crx", 2, 1},
    {"cry", 2, 1}, {"crz", 2, 1},  {"rxx", 2, 1},  {"rzz", 2, 1}, {"cu3", 2, 3}, {"ccx", 3, 0}, {"cswap", 3, 0},
};

const GateDef *lookup(const char *name) {
    for (const auto &g : kGates)
        if (!strcmp(g.name, name)) return &g;
    return nullptr;
}

constexpr double kPi2 = 1.57079632679489661923132169163975144;
constexpr double kPi4 = 0.785398163397448309615660845819875721;
constexpr double kSqrtHalf = 0.707106781186547524400844362104849039;

Mat u3(double th, double ph, double la) {
    const double ct = cos(th / 2.0), st = sin(th / 2.0);
    return {mk(ct, 0.0), scale(neg(expi(la)), st), scale(expi(ph), st), scale(expi(ph + la), ct)};
}
Mat rx(double th) {
    const double ct = cos(th / 2.0), st = sin(th / 2.0);
    return {mk(ct, 0.0), mk(0.0, -st), mk(0.0, -st), mk(ct, 0.0)};
}
Mat ry(double th) {
    const double ct = cos(th / 2.0), st = sin(th / 2.0);
    return {mk(ct, 0.0), mk(-st, 0.0), mk(st, 0.0), mk(ct, 0.0)};
}
Mat rz(double th) { return {expi(-th / 2.0), expi(th / 2.0)}; }
// Controlled 1-qubit unitary, qubits = [control, target] (control = bit 0).
Mat ctrl(const Mat &u) {
    Mat m(16);
    for (int j = 0; j < 4; j++) {
        if ((j & 1) == 0) {
            m[j * 4 + j] = mk(1.0, 0.0);
            continue;
        }
        const int t = (j >> 1) & 1;
        for (int tp = 0; tp < 2; tp++) m[(1 | (tp << 1)) * 4 + j] = u[tp * 2 + t];
    }
    return m;
}
template <typename F>
Mat perm(int dim, F f) {
    Mat m(dim * dim);
    for (int j = 0; j < dim; j++) m[f(j) * dim + j] = mk(1.0, 0.0);
    return m;
}

// Returns false for an unknown gate or a wrong parameter count.
bool build_gate(const std::string &n, const double *p, int np, bool *diag, Mat *out) {
    const GateDef *d = lookup(n.c_str());
    if (!d || d->nparams != np) return false;
    const Cx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    const double sq = kSqrtHalf;
    *diag = false;
    if (n == "id" || n == "u0") *diag = true, *out = {one, one};
    else if (n == "x") *out = {zero, one, one, zero};
    else if (n == "y") *out = {zero, mk(0.0, -1.0), mk(0.0, 1.0), zero};
    else if (n == "z") *diag = true, *out = {one, mk(-1.0, 0.0)};
    else if (n == "h") *out = {mk(sq, 0.0), mk(sq, 0.0), mk(sq, 0.0), mk(-sq, 0.0)};
    else if (n == "s") *diag = true, *out = {one, mk(0.0, 1.0)};
    else if (n == "sdg") *diag = true, *out = {one, mk(0.0, -1.0)};
    else if (n == "t") *diag = true, *out = {one, expi(kPi4)};
    else if (n == "tdg") *diag = true, *out = {one, expi(-kPi4)};
    else if (n == "sx") *out = {mk(0.5, 0.5), mk(0.5, -0.5), mk(0.5, -0.5), mk(0.5, 0.5)};
    else if (n == "sxdg") *out = {mk(0.5, -0.5), mk(0.5, 0.5), mk(0.5, 0.5), mk(0.5, -0.5)};
    else if (n == "rx") *out = rx(p[0]);
    else if (n == "ry") *out = ry(p[0]);
    else if (n == "rz") *diag = true, *out = rz(p[0]);
    else if (n == "u1" || n == "p") *diag = true, *out = {one, expi(p[0])};
    else if (n == "u2") *out = u3(kPi2, p[0], p[1]);
    else if (n == "u3" || n == "u") *out = u3(p[0], p[1], p[2]);
    else if (n == "cx") *out = perm(4, [](int j) { return (j & 1) ? j ^ 2 : j; });
    else if (n == "cy") *out = ctrl({zero, mk(0.0, -1.0), mk(0.0, 1.0), zero});
    else if (n == "cz") *diag = true, *out = {one, one, one, mk(-1.0, 0.0)};
    else if (n == "ch") *out = ctrl({mk(sq, 0.0), mk(sq, 0.0), mk(sq, 0.0), mk(-sq, 0.0)});
    else if (n == "swap") *out = perm(4, [](int j) { return ((j & 1) << 1) | ((j >> 1) & 1); });
    else if (n == "cp" || n == "cu1") *diag = true, *out = {one, one, one, expi(p[0])};
    else if (n == "crx") *out = ctrl(rx(p[0]));
    else if (n == "cry") *out = ctrl(ry(p[0]));
    else if (n == "crz") {
        Mat r = rz(p[0]);
        *diag = true, *out = {one, r[0], one, r[1]};
    } else if (n == "cu3") *out = ctrl(u3(p[0], p[1], p[2]));
    else if (n == "rxx") {
        const double ct = cos(p[0] / 2.0), st = sin(p[0] / 2.0);
        Mat m(16);
        for (int j = 0; j < 4; j++) {
            m[j * 4 + j] = mk(ct, 0.0);
            m[(j ^ 3) * 4 + j] = mk(0.0, -st);
        }
        *out = m;
    } else if (n == "rzz") {
        const Cx e0 = expi(-p[0] / 2.0), e1 = expi(p[0] / 2.0);
        *diag = true, *out = {e0, e1, e1, e0};
    } else if (n == "ccx") *out = perm(8, [](int j) { return (j & 3) == 3 ? j ^ 4 : j; });
    else if (n == "cswap")
        *out = perm(8, [](int j) { return (j & 1) ? ((j & 1) | ((j & 2) << 1) | ((j & 4) >> 1)) : j; });
    else return false;
    return true;
}

// ------------------------------------------------------------------ ops

struct Op {
    int kind = ZC_OP_UNITARY;
    std::vector<uint32_t> qs;  // sorted support (unitary / diagonal)
    Mat data;
    uint32_t a = 0, b = 0;     // CX (control, target), SWAP, measure (qubit, clbit), reset (qubit)
    bool has_if = false;
    uint32_t creg_offset = 0, creg_len = 0;
    uint64_t value = 0;

    // Qubits of a gate-like op (COp::gate_support); empty for others.
    std::vector<uint32_t> support() const {
        if (has_if) return {};
        if (kind == ZC_OP_UNITARY || kind == ZC_OP_DIAG) return qs;
        if (kind == ZC_OP_CX || kind == ZC_OP_SWAP) return {a, b};
        return {};
    }
    bool gate_like() const {
        return !has_if && (kind == ZC_OP_UNITARY || kind == ZC_OP_DIAG || kind == ZC_OP_CX || kind == ZC_OP_SWAP);
    }
};

// Local index over a sorted support -> the gate's argument-order index.
size_t to_arg_order(size_t j, const std::vector<int> &pos) {
    size_t r = 0;
    for (size_t b = 0; b < pos.size(); b++) r |= ((j >> pos[b]) & 1) << b;
    return r;
}

// Re-express a gate given in argument order on sorted qubits
// (permute_unitary_to_sorted / permute_diag_to_sorted).
void to_sorted(const std::vector<uint32_t> &args, const Mat &m, bool diag, std::vector<uint32_t> *sorted, Mat *out) {
    *sorted = args;
    std::sort(sorted->begin(), sorted->end());
    if (*sorted == args) {
        *out = m;
        return;
    }
    std::vector<int> pos(args.size());
    for (size_t b = 0; b < args.size(); b++)
        pos[b] = (int)(std::find(sorted->begin(), sorted->end(), args[b]) - sorted->begin());
    const size_t dim = (size_t)1 << args.size();
    out->assign(diag ? dim : dim * dim, Cx{});
    if (diag) {
        for (size_t j = 0; j < dim; j++) (*out)[j] = m[to_arg_order(j, pos)];
        return;
    }
    for (size_t i = 0; i < dim; i++) {
        const size_t ia = to_arg_order(i, pos);
        for (size_t j = 0; j < dim; j++) (*out)[i * dim + j] = m[ia * dim + to_arg_order(j, pos)];
    }
}

std::vector<uint32_t> merge(const std::vector<uint32_t> &x, const std::vector<uint32_t> &y) {
    std::vector<uint32_t> u(x);
    u.insert(u.end(), y.begin(), y.end());
    std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    return u;
}

// Index over `sub` (sorted) of the element with index i over `sup`.
size_t project(size_t i, const std::vector<uint32_t> &sub, const std::vector<uint32_t> &sup) {
    size_t j = 0;
    for (size_t b = 0; b < sub.size(); b++) {
        const size_t p = std::find(sup.begin(), sup.end(), sub[b]) - sup.begin();
        j |= ((i >> p) & 1) << b;
    }
    return j;
}

Mat widen_diag(const Mat &d, const std::vector<uint32_t> &from, const std::vector<uint32_t> &to) {
    if (from == to) return d;
    Mat out((size_t)1 << to.size());
    for (size_t i = 0; i < out.size(); i++) out[i] = d[project(i, from, to)];
    return out;
}

// Identity on the qubits of `to` outside `from` (embed_unitary).
Mat widen_unitary(const Mat &m, const std::vector<uint32_t> &from, const std::vector<uint32_t> &to) {
    if (from == to) return m;
    const size_t dt = (size_t)1 << to.size(), df = (size_t)1 << from.size();
    size_t fmask = 0;
    for (uint32_t q : from) fmask |= (size_t)1 << (std::find(to.begin(), to.end(), q) - to.begin());
    const size_t rest = (dt - 1) & ~fmask;
    Mat out(dt * dt);
    for (size_t i = 0; i < dt; i++) {
        const size_t fi = project(i, from, to);
        for (size_t j = 0; j < dt; j++) {
            if ((j & rest) != (i & rest)) continue;
            out[i * dt + j] = m[fi * df + project(j, from, to)];
        }
    }
    return out;
}

// a . b (row-major, dim x dim), accumulated i, l, j with zero a-entries
// skipped (matmul, src/compiler.rs:457-471).
Mat product(const Mat &a, const Mat &b, size_t dim) {
    Mat out(dim * dim);
    for (size_t i = 0; i < dim; i++)
        for (size_t l = 0; l < dim; l++) {
            const Cx ail = a[i * dim + l];
            if (is_zero(ail)) continue;
            for (size_t j = 0; j < dim; j++) out[i * dim + j] = out[i * dim + j] + ail * b[l * dim + j];
        }
    return out;
}

Mat dense_of(const Op &op, std::vector<uint32_t> *sup) {
    if (op.kind == ZC_OP_UNITARY) {
        *sup = op.qs;
        return op.data;
    }
    if (op.kind == ZC_OP_DIAG) {
        *sup = op.qs;
        const size_t dim = op.data.size();
        Mat m(dim * dim);
        for (size_t j = 0; j < dim; j++) m[j * dim + j] = op.data[j];
        return m;
    }
    Mat g;
    bool diag;
    build_gate(op.kind == ZC_OP_CX ? "cx" : "swap", nullptr, 0, &diag, &g);
    Mat out;
    to_sorted({op.a, op.b}, g, false, sup, &out);
    return out;
}

// fuse_diagonals (src/compiler.rs:477-535).
std::vector<Op> fuse_diagonals(std::vector<Op> ops, size_t diag_max) {
    std::vector<Op> out;
    bool have = false;
    Op cur;
    uint64_t blocked = 0;
    auto flush = [&]() {
        if (have) out.push_back(std::move(cur));
        have = false;
        blocked = 0;
    };
    for (Op &op : ops) {
        if (op.kind == ZC_OP_DIAG && !op.has_if) {
            bool clean = true;
            for (uint32_t q : op.qs) clean &= !((blocked >> q) & 1);
            if (have && clean) {
                std::vector<uint32_t> u = merge(cur.qs, op.qs);
                if (u.size() <= diag_max) {
                    Mat x = widen_diag(cur.data, cur.qs, u), y = widen_diag(op.data, op.qs, u);
                    for (size_t i = 0; i < x.size(); i++) x[i] = x[i] * y[i];
                    cur.data = std::move(x);
                    cur.qs = std::move(u);
                    continue;
                }
            }
            flush();
            cur = std::move(op);
            have = true;
        } else if (op.gate_like()) {
            if (have) {
                const std::vector<uint32_t> s = op.support();
                bool overlap = false;
                for (uint32_t q : s) overlap |= std::find(cur.qs.begin(), cur.qs.end(), q) != cur.qs.end();
                if (overlap) {
                    flush();
                } else {
                    for (uint32_t q : s) blocked |= 1ull << q;
                }
            }
            out.push_back(std::move(op));
        } else {
            flush();
            out.push_back(std::move(op));
        }
    }
    flush();
    return out;
}

// fuse_general (src/compiler.rs:540-626).
std::vector<Op> fuse_general(std::vector<Op> ops, size_t kmax) {
    std::vector<Op> out;
    bool have = false;
    std::vector<uint32_t> gsup;
    Mat gmat;
    size_t count = 0;
    Op first;
    auto flush = [&]() {
        if (!have) return;
        if (count == 1) {
            out.push_back(std::move(first));
        } else {
            Op f;
            f.kind = ZC_OP_UNITARY;
            f.qs = gsup;
            f.data = std::move(gmat);
            out.push_back(std::move(f));
        }
        have = false;
    };
    for (Op &op : ops) {
        const std::vector<uint32_t> s = op.support();
        if (!op.gate_like() || s.size() > kmax) {
            flush();
            out.push_back(std::move(op));
            continue;
        }
        if (have) {
            std::vector<uint32_t> qs;
            Mat m = dense_of(op, &qs);
            std::vector<uint32_t> u = merge(gsup, qs);
            if (u.size() <= kmax) {
                gmat = product(widen_unitary(m, qs, u), widen_unitary(gmat, gsup, u), (size_t)1 << u.size());
                gsup = std::move(u);
                count++;
                continue;
            }
            flush();
        }
        gmat = dense_of(op, &gsup);
        count = 1;
        first = std::move(op);
        have = true;
    }
    flush();
    return out;
}

const char *kSelfInverse[] = {"x", "y", "z", "h", "cx", "cy", "cz", "ch", "swap", "ccx", "cswap"};

bool self_inverse(const char *n) {
    for (const char *s : kSelfInverse)
        if (!strcmp(s, n)) return true;
    return false;
}

bool plain_gate(const zc_instr &i) { return i.kind == ZC_I_GATE && i.cond_creg < 0; }

bool same_gate(const zc_instr &x, const zc_instr &y) {
    if (strncmp(x.name, y.name, 8) || x.nq != y.nq) return false;
    for (uint32_t i = 0; i < x.nq; i++)
        if (x.q[i] != y.q[i]) return false;
    return true;
}

bool overlaps(const zc_instr &x, const zc_instr &y) {
    for (uint32_t i = 0; i < x.nq; i++)
        for (uint32_t j = 0; j < y.nq; j++)
            if (x.q[i] == y.q[j]) return true;
    return false;
}

// cancel (src/compiler.rs:215-239): drop adjacent self-inverse pairs,
// looking back through gates on disjoint qubits; non-gates fence.
std::vector<zc_instr> cancel_pairs(const zc_instr *ins, size_t n) {
    std::vector<zc_instr> out;
    out.reserve(n);
    for (size_t x = 0; x < n; x++) {
        const zc_instr &g = ins[x];
        char name[9] = {0};
        memcpy(name, g.name, 8);
        bool dropped = false;
        if (plain_gate(g) && g.np == 0 && self_inverse(name)) {
            for (size_t i = out.size(); i-- > 0;) {
                if (!plain_gate(out[i])) break;
                if (!overlaps(out[i], g)) continue;
                if (same_gate(out[i], g)) {
                    out.erase(out.begin() + (long)i);
                    dropped = true;
                }
                break;
            }
        }
        if (!dropped) out.push_back(g);
    }
    return out;
}

}  // namespace
}  // namespace zc

struct zc_program {
    uint32_t n_qubits = 0, n_clbits = 0;
    std::vector<zc::Op> ops;
    bool dynamic = false;
    std::vector<std::pair<uint32_t, uint32_t>> finals;
    zc_program_info info{};
    std::vector<std::vector<double>> views;  // interleaved copies for zc_program_get_op
};

namespace zc {
namespace {

int lower_instr(const zc_instr &g, uint32_t nq, uint32_t ncl, const uint32_t *cregs, uint32_t ncregs,
                bool swap_perm, std::vector<Op> *out) {
    char name[9] = {0};
    memcpy(name, g.name, 8);
    Op op;
    bool emit = true;
    char buf[200];
    if (g.kind == ZC_I_GATE) {
        const GateDef *d = lookup(name);
        if (!d) {
            snprintf(buf, sizeof buf, "invalid circuit: unknown gate '%s'", name);
            return fail(ZC_ERR_INVALID, buf);
        }
        if ((int)g.nq != d->arity) {
            snprintf(buf, sizeof buf, "invalid circuit: gate '%s' expects %d qubit(s), got %u", name, d->arity, g.nq);
            return fail(ZC_ERR_INVALID, buf);
        }
        for (uint32_t i = 0; i < g.nq; i++)
            if (g.q[i] >= nq) {
                snprintf(buf, sizeof buf, "invalid circuit: qubit %u out of range (have %u)", g.q[i], nq);
                return fail(ZC_ERR_INVALID, buf);
            }
        for (uint32_t i = 0; i < g.nq; i++)
            for (uint32_t j = i + 1; j < g.nq; j++)
                if (g.q[i] == g.q[j]) {
                    snprintf(buf, sizeof buf, "invalid circuit: gate '%s' applied to duplicate qubits", name);
                    return fail(ZC_ERR_INVALID, buf);
                }
        const std::string n(name);
        if (n == "id" || n == "u0") {
            emit = false;
        } else if (n == "cx") {
            op.kind = ZC_OP_CX;
            op.a = g.q[0];
            op.b = g.q[1];
        } else if (n == "swap" && swap_perm) {
            op.kind = ZC_OP_SWAP;
            op.a = std::min(g.q[0], g.q[1]);
            op.b = std::max(g.q[0], g.q[1]);
        } else {
            Mat m;
            bool diag;
            if (!build_gate(n, g.p, (int)g.np, &diag, &m)) {
                snprintf(buf, sizeof buf, "invalid circuit: gate '%s' expects %d parameter(s), got %u", name,
                         d->nparams, g.np);
                return fail(ZC_ERR_INVALID, buf);
            }
            op.kind = diag ? ZC_OP_DIAG : ZC_OP_UNITARY;
            to_sorted(std::vector<uint32_t>(g.q, g.q + g.nq), m, diag, &op.qs, &op.data);
        }
    } else if (g.kind == ZC_I_MEASURE || g.kind == ZC_I_RESET) {
        if (g.q[0] >= nq) {
            snprintf(buf, sizeof buf, "invalid circuit: qubit %u out of range (have %u)", g.q[0], nq);
            return fail(ZC_ERR_INVALID, buf);
        }
        if (g.kind == ZC_I_MEASURE && g.clbit >= ncl) {
            snprintf(buf, sizeof buf, "invalid circuit: clbit %u out of range (have %u)", g.clbit, ncl);
            return fail(ZC_ERR_INVALID, buf);
        }
        op.kind = g.kind == ZC_I_MEASURE ? ZC_OP_MEASURE : ZC_OP_RESET;
        op.a = g.q[0];
        op.b = g.clbit;
    } else {
        op.kind = -1;  // barrier: fusion fence, stripped after fusion
    }
    if (!emit) return ZC_OK;
    if (g.cond_creg >= 0) {
        if ((uint32_t)g.cond_creg >= ncregs) return fail(ZC_ERR_INVALID, "invalid circuit: creg out of range");
        op.has_if = true;
        for (int i = 0; i < g.cond_creg; i++) op.creg_offset += cregs[i];
        op.creg_len = cregs[g.cond_creg];
        op.value = g.cond_value;
    }
    out->push_back(std::move(op));
    return ZC_OK;
}

// ------------------------------------------------------------------ executor

int apply_gate_op(zc_state *st, const Op &op) {
    switch (op.kind) {
        case ZC_OP_UNITARY:
            return zc_apply_unitary(st, op.qs.data(), (uint32_t)op.qs.size(), (const double *)op.data.data());
        case ZC_OP_DIAG:
            return zc_apply_diagonal(st, op.qs.data(), (uint32_t)op.qs.size(), (const double *)op.data.data());
        case ZC_OP_CX:
            return zc_apply_cx(st, op.a, op.b);
        case ZC_OP_SWAP:
            return zc_apply_swap(st, op.a, op.b);
        default:
            return fail(ZC_ERR_INVALID, "non-unitary op in a static body");
    }
}

// apply_pauli (src/noise.rs:91-100): 1 = X, 2 = Y, 3 = Z.
int apply_pauli(zc_state *st, uint32_t q, uint64_t code) {
    static const double X[8] = {0, 0, 1, 0, 1, 0, 0, 0};
    static const double Y[8] = {0, 0, 0, -1, 0, 1, 0, 0};
    static const double Z[4] = {1, 0, -1, 0};
    if (code == 1) return zc_apply_unitary(st, &q, 1, X);
    if (code == 2) return zc_apply_unitary(st, &q, 1, Y);
    if (code == 3) return zc_apply_diagonal(st, &q, 1, Z);
    return ZC_OK;
}

// amplitude_damp (src/noise.rs:114-127).
int amplitude_damp(zc_state *st, uint32_t q, double gamma, double u) {
    double p1 = 0.0;
    int rc = zc_prob_one(st, q, &p1);
    if (rc) return rc;
    const double p_jump = gamma * p1;
    if (u < p_jump) {
        int o = 0;
        rc = zc_measure(st, q, 0.0, &o);
        if (rc) return rc;
        return apply_pauli(st, q, 1);
    }
    const double s = 1.0 / sqrt(1.0 - p_jump);
    const double d[4] = {s, 0.0, s * sqrt(1.0 - gamma), 0.0};
    return zc_apply_diagonal(st, &q, 1, d);
}

// apply_gate_noise (src/noise.rs:145-175): frozen channel and draw order.
int gate_noise(zc_state *st, const zc_noise &m, const std::vector<uint32_t> &qs, Xoshiro &rng) {
    const uint32_t k = (uint32_t)qs.size();
    const double p_dep = k == 1 ? m.depolarizing_1q : m.depolarizing_2q;
    int rc = ZC_OK;
    if (p_dep > 0.0 && rng.f64() < p_dep) {
        const uint64_t idx = rng.range(1, 1ull << (2 * k));
        for (uint32_t b = 0; b < k; b++)
            if ((rc = apply_pauli(st, qs[b], (idx >> (2 * b)) & 3))) return rc;
    }
    for (uint32_t q : qs) {
        if (m.bit_flip > 0.0 && rng.f64() < m.bit_flip && (rc = apply_pauli(st, q, 1))) return rc;
        if (m.phase_flip > 0.0 && rng.f64() < m.phase_flip && (rc = apply_pauli(st, q, 3))) return rc;
        if (m.amplitude_damping > 0.0) {
            const double u = rng.f64();
            if ((rc = amplitude_damp(st, q, m.amplitude_damping, u))) return rc;
        }
    }
    return ZC_OK;
}

bool readout_flip(const zc_noise &m, bool bit, Xoshiro &rng) {
    const double p = bit ? m.readout_flip_1to0 : m.readout_flip_0to1;
    if (p > 0.0 && rng.f64() < p) return !bit;
    return bit;
}

bool trivial(const zc_noise *m) {
    return !m || (m->depolarizing_1q == 0.0 && m->depolarizing_2q == 0.0 && m->bit_flip == 0.0 &&
                  m->phase_flip == 0.0 && m->amplitude_damping == 0.0 && m->readout_flip_0to1 == 0.0 &&
                  m->readout_flip_1to0 == 0.0);
}

// NoiseModel::validate (src/noise.rs:77-87): every field a probability in
// [0, 1]; NaN is rejected.
int validate_noise(const zc_noise &m) {
    const std::pair<const char *, double> fields[] = {
        {"depolarizing_1q", m.depolarizing_1q},     {"depolarizing_2q", m.depolarizing_2q},
        {"bit_flip", m.bit_flip},                   {"phase_flip", m.phase_flip},
        {"amplitude_damping", m.amplitude_damping}, {"readout_flip_0to1", m.readout_flip_0to1},
        {"readout_flip_1to0", m.readout_flip_1to0}};
    for (const auto &f : fields)
        if (!(f.second >= 0.0 && f.second <= 1.0)) {
            char buf[128];
            if (std::isnan(f.second))
                snprintf(buf, sizeof buf, "%s = NaN is not a probability in [0, 1]", f.first);
            else
                snprintf(buf, sizeof buf, "%s = %g is not a probability in [0, 1]", f.first, f.second);
            return fail(ZC_ERR_INVALID, buf);
        }
    return ZC_OK;
}

// exec_shot_op (src/exec.rs:556-619).
int shot_op(zc_state *st, const Op &op, const zc_noise *noise, Xoshiro &rng, uint64_t *clbits) {
    if (op.has_if) {
        const uint64_t mask = op.creg_len >= 64 ? ~0ull : ((1ull << op.creg_len) - 1);
        if (((*clbits >> op.creg_offset) & mask) != op.value) return ZC_OK;
    }
    int rc = ZC_OK;
    switch (op.kind) {
        case ZC_OP_UNITARY:
        case ZC_OP_DIAG:
            if ((rc = apply_gate_op(st, op))) return rc;
            if (noise) return gate_noise(st, *noise, op.qs, rng);
            return ZC_OK;
        case ZC_OP_CX:
        case ZC_OP_SWAP:
            if ((rc = apply_gate_op(st, op))) return rc;
            if (noise) return gate_noise(st, *noise, {std::min(op.a, op.b), std::max(op.a, op.b)}, rng);
            return ZC_OK;
        case ZC_OP_MEASURE: {
            int bit = 0;
            if ((rc = zc_measure(st, op.a, rng.f64(), &bit))) return rc;
            if (noise) bit = readout_flip(*noise, bit != 0, rng);
            *clbits = (*clbits & ~(1ull << op.b)) | ((uint64_t)(bit != 0) << op.b);
            return ZC_OK;
        }
        case ZC_OP_RESET: {
            int bit = 0;
            if ((rc = zc_measure(st, op.a, rng.f64(), &bit))) return rc;
            if (bit) return apply_pauli(st, op.a, 1);
            return ZC_OK;
        }
        default:
            return ZC_OK;
    }
}

void histogram(std::vector<uint64_t> &w, std::vector<std::pair<uint64_t, uint64_t>> *out) {
    std::sort(w.begin(), w.end());
    for (size_t i = 0; i < w.size();) {
        size_t j = i;
        while (j < w.size() && w[j] == w[i]) j++;
        out->push_back({w[i], (uint64_t)(j - i)});
        i = j;
    }
}

// Can the batched trajectory engine run this noisy program?
bool batchable(const zc_program *p) {
    for (const Op &o : p->ops) {
        const bool gate = o.kind == ZC_OP_UNITARY || o.kind == ZC_OP_DIAG || o.kind == ZC_OP_CX || o.kind == ZC_OP_SWAP;
        if (!gate && o.kind != ZC_OP_MEASURE && o.kind != ZC_OP_RESET) return false;
        if ((o.kind == ZC_OP_UNITARY || o.kind == ZC_OP_DIAG) && o.qs.size() > 3) return false;
    }
    return p->n_clbits <= 64;  // one classical word per trajectory, as the per-shot path
}

// Noisy or dynamic program, all shots as trajectories in one launch.
int run_batched(const zc_program *p, const zc_run_options *opt, const zc_noise &nz,
                std::vector<std::pair<uint64_t, uint64_t>> *hist, zc_run_result *res) {
    std::vector<TrajOp> tops;
    std::vector<double> mats = {1, 0, 0, 0, 0, 0, 1, 0};  // 2x2 identity for measure / reset
    for (const Op &o : p->ops) {
        TrajOp t{};
        if (o.kind == ZC_OP_MEASURE || o.kind == ZC_OP_RESET) {
            t.k = 1;
            t.qs[0] = o.a;
            t.kind = o.kind == ZC_OP_MEASURE ? TOP_MEASURE : TOP_RESET;
            t.clbit = o.b;
            t.mat_off = 0;
        } else {
            std::vector<uint32_t> sup;
            Mat m = dense_of(o, &sup);
            t.k = (uint32_t)sup.size();
            for (size_t i = 0; i < sup.size(); i++) t.qs[i] = sup[i];
            t.kind = TOP_GATE;
            t.mat_off = (uint32_t)mats.size();
            for (const Cx &c : m) {
                mats.push_back(c.re);
                mats.push_back(c.im);
            }
        }
        if (o.has_if) {
            t.cond = 1;
            t.cond_off = o.creg_offset;
            t.cond_len = o.creg_len;
            t.cond_value = o.value;
        }
        tops.push_back(t);
    }
    std::vector<uint32_t> fq, fc;
    for (const auto &f : p->finals) {
        fq.push_back(f.first);
        fc.push_back(f.second);
    }
    TrajNoise tn{{nz.depolarizing_1q, nz.depolarizing_2q, nz.bit_flip, nz.phase_flip, nz.amplitude_damping,
                  nz.readout_flip_0to1, nz.readout_flip_1to0}};
    zc_state *ctx = nullptr;
    int rc = zc_create_ex(1, 32, opt->flags, &ctx);
    if (rc) return rc;
    const uint64_t ntraj = opt->shots;
    const size_t per_cta = ((size_t)2 << p->n_qubits) * sizeof(float);
    uint64_t budget = 0;
    zc_device_budget(opt->mem_fraction > 0 ? opt->mem_fraction : 0.75, &budget);
    uint64_t ctas = std::min<uint64_t>(ntraj, (uint64_t)ctx->num_sms * 4);  // four trajectories per SM
    ctas = std::min<uint64_t>(ctas, std::max<uint64_t>(1, budget / std::max<size_t>(per_cta, 1)));
    void *d_work = nullptr, *d_buf = nullptr;
    const size_t ops_b = tops.size() * sizeof(TrajOp), mats_b = mats.size() * sizeof(double);
    const size_t f_b = (fq.size() + 1) * sizeof(uint32_t), out_b = ntraj * sizeof(uint64_t);
    const size_t off_mats = (ops_b + 255) & ~(size_t)255, off_fq = off_mats + ((mats_b + 255) & ~(size_t)255);
    const size_t off_fc = off_fq + ((f_b + 255) & ~(size_t)255), off_out = off_fc + ((f_b + 255) & ~(size_t)255);
    std::vector<uint64_t> words(ntraj);
    auto cleanup = [&](int code) {
        if (d_work) cudaFree(d_work);
        if (d_buf) cudaFree(d_buf);
        zc_counters c{};
        zc_get_counters(ctx, &c);
        res->launches = c.launches;
        zc_destroy(ctx);
        return code;
    };
    cudaError_t e = cudaMalloc(&d_work, per_cta * ctas);
    if (e == cudaSuccess) e = cudaMalloc(&d_buf, off_out + out_b);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "cudaMalloc (trajectory buffers)"));
    char *b = (char *)d_buf;
    cudaStream_t s = ctx->stream;
    if (!tops.empty()) cudaMemcpyAsync(b, tops.data(), ops_b, cudaMemcpyHostToDevice, s);
    if (!mats.empty()) cudaMemcpyAsync(b + off_mats, mats.data(), mats_b, cudaMemcpyHostToDevice, s);
    if (!fq.empty()) {
        cudaMemcpyAsync(b + off_fq, fq.data(), fq.size() * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(b + off_fc, fc.data(), fc.size() * 4, cudaMemcpyHostToDevice, s);
    }
    rc = launch_trajectories(ctx, p->n_qubits, (const TrajOp *)b, (int)tops.size(), (const double *)(b + off_mats),
                             (const uint32_t *)(b + off_fq), (const uint32_t *)(b + off_fc), (int)fq.size(), tn, ntraj,
                             opt->seed, (uint64_t *)(b + off_out), d_work, (int)ctas);
    if (rc) return cleanup(rc);
    e = cudaMemcpyAsync(words.data(), b + off_out, out_b, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cleanup(cuda_fail(e, "trajectory launch"));
    histogram(words, hist);
    res->batched = 1;
    return cleanup(ZC_OK);
}

}  // namespace
}  // namespace zc

using namespace zc;

extern "C" {

int zc_compile(uint32_t nq, const uint32_t *cregs, uint32_t ncregs, const zc_instr *ins, size_t n_ins,
               const zc_compile_options *opt_in, zc_program **out) {
    if (!out) return fail(ZC_ERR_INVALID, "null output");
    *out = nullptr;
    zc_compile_options opt = opt_in ? *opt_in : zc_compile_options{1, 10, 1};
    uint32_t ncl = 0;
    for (uint32_t i = 0; i < ncregs; i++) ncl += cregs[i];
    if (nq == 0) return fail(ZC_ERR_INVALID, "invalid circuit: no qubits declared");
    if (nq > 48) return fail(ZC_ERR_INVALID, "invalid circuit: too many qubits for any state-vector budget");
    if (ncl > 64) return fail(ZC_ERR_INVALID, "invalid circuit: more than 64 classical bits are not supported");
    size_t input_gates = 0;
    for (size_t i = 0; i < n_ins; i++) input_gates += ins[i].kind == ZC_I_GATE;
    std::vector<zc_instr> kept = cancel_pairs(ins, n_ins);
    size_t kept_gates = 0;
    for (const auto &i : kept) kept_gates += i.kind == ZC_I_GATE;
    std::vector<Op> ops;
    for (const auto &i : kept) {
        int rc = lower_instr(i, nq, ncl, cregs, ncregs, opt.swap_perm != 0, &ops);
        if (rc) return rc;
    }
    const size_t kmax = std::min<uint32_t>(opt.fusion_max, kMaxUnitaryQubits);
    const size_t dmax = std::min<uint32_t>(opt.diag_max, kMaxDiagQubits);
    if (kmax >= 1) {
        ops = fuse_diagonals(std::move(ops), dmax);
        ops = fuse_general(std::move(ops), kmax);
    }
    ops.erase(std::remove_if(ops.begin(), ops.end(), [](const Op &o) { return o.kind == -1; }), ops.end());
    zc_program *p = new zc_program();
    p->n_qubits = nq;
    p->n_clbits = ncl;
    size_t split = ops.size();
    while (split > 0 && ops[split - 1].kind == ZC_OP_MEASURE && !ops[split - 1].has_if) split--;
    for (size_t i = 0; i < split; i++)
        if (ops[i].has_if || ops[i].kind == ZC_OP_MEASURE || ops[i].kind == ZC_OP_RESET) p->dynamic = true;
    if (!p->dynamic) {
        for (size_t i = split; i < ops.size(); i++) p->finals.push_back({ops[i].a, ops[i].b});
        ops.resize(split);
    }
    size_t maxf = 0;
    for (const Op &o : ops) maxf = std::max(maxf, o.support().size());
    p->ops = std::move(ops);
    p->info = zc_program_info{nq, ncl, p->ops.size(), p->finals.size(), p->dynamic,
                              input_gates, input_gates - kept_gates, p->ops.size(), maxf};
    p->views.resize(p->ops.size());
    *out = p;
    return ZC_OK;
}

void zc_program_free(zc_program *p) { delete p; }

int zc_program_get_info(const zc_program *p, zc_program_info *out) {
    if (!p || !out) return fail(ZC_ERR_INVALID, "null argument");
    *out = p->info;
    return ZC_OK;
}

int zc_program_get_op(const zc_program *p, size_t i, zc_op_view *v) {
    if (!p || !v || i >= p->ops.size()) return fail(ZC_ERR_INVALID, "bad op index");
    const Op &o = p->ops[i];
    memset(v, 0, sizeof *v);
    v->kind = o.kind;
    v->k = (uint32_t)o.qs.size();
    for (size_t j = 0; j < o.qs.size() && j < 12; j++) v->qubits[j] = o.qs[j];
    v->data = o.data.empty() ? nullptr : (const double *)o.data.data();
    v->a = o.a;
    v->b = o.b;
    v->has_if = o.has_if;
    v->creg_offset = o.creg_offset;
    v->creg_len = o.creg_len;
    v->value = o.value;
    return ZC_OK;
}

int zc_program_get_final(const zc_program *p, size_t i, uint32_t *q, uint32_t *c) {
    if (!p || i >= p->finals.size() || !q || !c) return fail(ZC_ERR_INVALID, "bad final-measure index");
    *q = p->finals[i].first;
    *c = p->finals[i].second;
    return ZC_OK;
}

int zc_run(const zc_program *p, const zc_run_options *opt, zc_run_result *res, uint64_t *keys, uint64_t *counts,
           size_t cap, double *sv) {
    if (!p || !opt || !res) return fail(ZC_ERR_INVALID, "null argument");
    memset(res, 0, sizeof *res);
    // run_inner (src/exec.rs:347-351): a non-trivial model is validated first
    const zc_noise *noise = trivial(opt->noise) ? nullptr : opt->noise;
    if (noise) {
        const int vrc = validate_noise(*noise);
        if (vrc) return vrc;
    }
    if ((noise || p->dynamic) && sv)
        return fail(ZC_ERR_INVALID, noise ? "a noise model is active: the noisy state has no single final state vector"
                                          : "circuit is dynamic: it has no single final state vector");
    // resolve_precision (src/exec.rs:261-304) against the HBM budget: an
    // explicit precision must fit; auto takes f64 if it fits, else f32 with
    // zeno's notice (and refuses if f32 does not fit either)
    uint64_t budget = 0;
    int rc = zc_device_budget(opt->mem_fraction > 0 ? opt->mem_fraction : 0.75, &budget);
    if (rc) return rc;
    int prec = opt->precision_bits;
    std::string notices;
    auto notice = [&](const std::string &s) { notices += s + "\n"; };
    if (prec != 0 && prec != 32 && prec != 64) return fail(ZC_ERR_INVALID, "precision_bits must be 0, 32 or 64");
    if (prec == 0) {
        if (zc_state_bytes(p->n_qubits, 64) <= budget) {
            prec = 64;
        } else {
            prec = 32;
            notice("auto-precision: " + std::to_string(p->n_qubits) +
                   " qubits exceed the f64 budget, using f32 (8 B/amplitude)");
        }
    }
    if ((rc = plan_state(p->n_qubits, prec, budget))) return rc;
    res->precision_bits = prec;
    // run_inner / run_sampled / run_per_shot notices (src/exec.rs:374, :429-435, :478-481)
    if (noise) notice("noise: trajectory sampling \xe2\x80\x94 per-shot execution, fusion disabled");
    if (!p->dynamic && p->finals.empty() && opt->shots > 0)
        notice(noise ? "circuit has no measurements: counts are empty"
                     : "circuit has no measurements: counts are empty (use --statevector to inspect the state)");
    auto put_notices = [&]() {
        const size_t n = std::min(notices.size(), sizeof(res->notices) - 1);
        memcpy(res->notices, notices.data(), n);
        res->notices[n] = 0;
    };
    put_notices();
    const auto t0 = std::chrono::steady_clock::now();
    if ((noise || p->dynamic) && prec == 32 && !(opt->flags & ZC_FLAG_PER_SHOT) && batchable(p)) {
        std::vector<std::pair<uint64_t, uint64_t>> hist;
        const zc_noise none{};
        rc = p->finals.empty() && !p->dynamic ? ZC_OK : run_batched(p, opt, noise ? *noise : none, &hist, res);
        res->sim_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        res->n_keys = hist.size();
        for (size_t i = 0; i < hist.size() && i < cap; i++) {
            keys[i] = hist[i].first;
            counts[i] = hist[i].second;
        }
        return rc;
    }
    zc_state *st = nullptr;
    rc = create_state(p->n_qubits, prec, opt->flags, budget, &st);
    if (rc) return rc;
    if (opt->sweep_high && (rc = zc_set_sweep_shape(st, opt->sweep_high))) {
        zc_destroy(st);
        return rc;
    }
    std::vector<std::pair<uint64_t, uint64_t>> hist;
    auto done = [&](int code) {
        if (st) {
            zc_counters c{};
            zc_get_counters(st, &c);
            res->launches = c.launches;
            res->sweeps = c.sweeps;
            res->bytes_moved = c.bytes_moved;
            zc_destroy(st);
        }
        return code;
    };
    if (!noise && !p->dynamic) {
        // run_sampled (src/exec.rs:407-452)
        for (const Op &op : p->ops)
            if ((rc = apply_gate_op(st, op))) return done(rc);
        if ((rc = zc_finish(st))) return done(rc);
        if (sv && (rc = zc_statevector(st, sv))) return done(rc);
        if (!p->finals.empty() && opt->shots > 0) {
            std::vector<uint64_t> idx(opt->shots);
            if ((rc = zc_sample(st, opt->shots, splitmix64(opt->seed), idx.data()))) return done(rc);
            for (uint64_t &b : idx) {
                uint64_t cl = 0;
                for (const auto &f : p->finals) cl = (cl & ~(1ull << f.second)) | (((b >> f.first) & 1) << f.second);
                b = cl;
            }
            histogram(idx, &hist);
        }
    } else if (p->dynamic || !p->finals.empty()) {
        // run_per_shot (src/exec.rs:459-549), one trajectory after another
        std::vector<uint64_t> words(opt->shots);
        for (uint64_t shot = 0; shot < opt->shots; shot++) {
            if ((rc = zc_reset_all(st))) return done(rc);
            Xoshiro rng(splitmix64(opt->seed ^ shot));
            uint64_t cl = 0;
            for (const Op &op : p->ops)
                if ((rc = shot_op(st, op, noise, rng, &cl))) return done(rc);
            for (const auto &f : p->finals) {
                int bit = 0;
                if ((rc = zc_measure(st, f.first, rng.f64(), &bit))) return done(rc);
                if (noise) bit = readout_flip(*noise, bit != 0, rng);
                cl = (cl & ~(1ull << f.second)) | ((uint64_t)(bit != 0) << f.second);
            }
            words[shot] = cl;
        }
        histogram(words, &hist);
    }
    rc = zc_finish(st);
    res->sim_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    res->n_keys = hist.size();
    for (size_t i = 0; i < hist.size() && i < cap; i++) {
        keys[i] = hist[i].first;
        counts[i] = hist[i].second;
    }
    return done(rc);
}

}  // extern "C"
