/*
 * zeno_oracle.c — CPU oracle (TEST INFRASTRUCTURE ONLY; see zeno_oracle.h).
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off, no fast-math). The
 * kernels keep the reference's exact expression trees and never contract
 * to FMA, so they reproduce the reference's scalar arithmetic bit for bit.
 * Each function cites the reference file:line it restates.
 */
#include "zeno_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ===================================================================== */
/* RNG: splitmix64 (src/exec.rs:227-232), xoshiro256++ seeded through     */
/* SplitMix64 (rand_xoshiro 0.6 seed_from_u64), rand 0.8 f64 / gen_range. */
/* ===================================================================== */

uint64_t zo_splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

void zo_rng_seed(zo_rng *r, uint64_t seed) {
    /* SplitMix64 state starts at `seed`; four outputs fill the 32-byte seed
     * little-endian, i.e. s[i] = i-th output. */
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) {
        x += 0x9E3779B97F4A7C15ULL;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        r->s[i] = z ^ (z >> 31);
    }
}

static inline uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

uint64_t zo_rng_next(zo_rng *r) {
    uint64_t *s = r->s;
    uint64_t result = rotl64(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl64(s[3], 45);
    return result;
}

double zo_rng_f64(zo_rng *r) {
    /* 53 high bits times 2^-53: uniform on [0, 1). */
    uint64_t v = zo_rng_next(r) >> 11;
    return (double)v * (1.0 / 9007199254740992.0);
}

uint64_t zo_rng_range(zo_rng *r, uint64_t lo, uint64_t hi) {
    /* Widening-multiply rejection with the "conservative zone" of rand 0.8's
     * UniformInt<u64>::sample_single_inclusive(lo, hi - 1). */
    uint64_t range = hi - lo; /* (hi-1) - lo + 1 */
    if (range == 0) return zo_rng_next(r);
    int lz = __builtin_clzll(range);
    uint64_t zone = (range << lz) - 1;
    for (;;) {
        uint64_t v = zo_rng_next(r);
        unsigned __int128 m = (unsigned __int128)v * range;
        uint64_t mlo = (uint64_t)m, mhi = (uint64_t)(m >> 64);
        if (mlo <= zone) return lo + mhi;
    }
}

/* ===================================================================== */
/* Complex helpers with num-complex 0.4 semantics.                        */
/* ===================================================================== */

static inline zo_c64 cx(double re, double im) {
    zo_c64 z = {re, im};
    return z;
}
static inline zo_c64 cmul(zo_c64 a, zo_c64 b) {
    return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline zo_c64 cadd(zo_c64 a, zo_c64 b) { return cx(a.re + b.re, a.im + b.im); }
static inline zo_c64 cscale(zo_c64 a, double s) { return cx(a.re * s, a.im * s); }
static inline zo_c64 cneg(zo_c64 a) { return cx(-a.re, -a.im); }
static inline zo_c64 expi(double t) { return cx(cos(t), sin(t)); }
static inline int ciszero(zo_c64 a) { return a.re == 0.0 && a.im == 0.0; }

/* ===================================================================== */
/* Gate library (src/gates.rs:101-188).                                   */
/* ===================================================================== */

static const double FRAC_PI_2_ = 1.57079632679489661923132169163975144;
static const double FRAC_PI_4_ = 0.785398163397448309615660845819875721;
static const double FRAC_1_SQRT_2_ = 0.707106781186547524400844362104849039;

int zo_gate_lookup(const char *name, int *arity, int *nparams) {
    static const struct {
        const char *n;
        int a, p;
    } tab[] = {
        {"id", 1, 0},   {"u0", 1, 0},   {"x", 1, 0},     {"y", 1, 0},    {"z", 1, 0},    {"h", 1, 0},
        {"s", 1, 0},    {"sdg", 1, 0},  {"t", 1, 0},     {"tdg", 1, 0},  {"sx", 1, 0},   {"sxdg", 1, 0},
        {"rx", 1, 1},   {"ry", 1, 1},   {"rz", 1, 1},    {"u1", 1, 1},   {"p", 1, 1},    {"u2", 1, 2},
        {"u3", 1, 3},   {"u", 1, 3},    {"cx", 2, 0},    {"cy", 2, 0},   {"cz", 2, 0},   {"ch", 2, 0},
        {"swap", 2, 0}, {"cp", 2, 1},   {"cu1", 2, 1},   {"crx", 2, 1},  {"cry", 2, 1},  {"crz", 2, 1},
        {"rxx", 2, 1},  {"rzz", 2, 1},  {"cu3", 2, 3},   {"ccx", 3, 0},  {"cswap", 3, 0},
    };
    for (size_t i = 0; i < sizeof(tab) / sizeof(tab[0]); i++) {
        if (strcmp(tab[i].n, name) == 0) {
            if (arity) *arity = tab[i].a;
            if (nparams) *nparams = tab[i].p;
            return 1;
        }
    }
    return 0;
}

static void u3m(double th, double ph, double la, zo_c64 *m) {
    double ct = cos(th / 2.0), st = sin(th / 2.0);
    m[0] = cx(ct, 0.0);
    m[1] = cscale(cneg(expi(la)), st);
    m[2] = cscale(expi(ph), st);
    m[3] = cscale(expi(ph + la), ct);
}
static void rxm(double th, zo_c64 *m) {
    double ct = cos(th / 2.0), st = sin(th / 2.0);
    m[0] = cx(ct, 0.0);
    m[1] = cx(0.0, -st);
    m[2] = cx(0.0, -st);
    m[3] = cx(ct, 0.0);
}
static void rym(double th, zo_c64 *m) {
    double ct = cos(th / 2.0), st = sin(th / 2.0);
    m[0] = cx(ct, 0.0);
    m[1] = cx(-st, 0.0);
    m[2] = cx(st, 0.0);
    m[3] = cx(ct, 0.0);
}
static void rz_diag(double th, zo_c64 *d) {
    d[0] = expi(-th / 2.0);
    d[1] = expi(th / 2.0);
}
static void controlled1(const zo_c64 *u, zo_c64 *m) {
    for (int i = 0; i < 16; i++) m[i] = cx(0, 0);
    for (int j = 0; j < 4; j++) {
        int ctrl = j & 1, t = (j >> 1) & 1;
        if (ctrl == 0) {
            m[j * 4 + j] = cx(1.0, 0.0);
        } else {
            for (int tp = 0; tp < 2; tp++) {
                int i = 1 | (tp << 1);
                m[i * 4 + j] = u[tp * 2 + t];
            }
        }
    }
}
static void permutation(int dim, int (*perm)(int), zo_c64 *m) {
    for (int i = 0; i < dim * dim; i++) m[i] = cx(0, 0);
    for (int j = 0; j < dim; j++) m[perm(j) * dim + j] = cx(1.0, 0.0);
}
static int perm_cx(int j) { return (j & 1) ? (j ^ 2) : j; }
static int perm_swap(int j) { return ((j & 1) << 1) | ((j >> 1) & 1); }
static int perm_ccx(int j) { return ((j & 3) == 3) ? (j ^ 4) : j; }
static int perm_cswap(int j) { return (j & 1) ? ((j & 1) | ((j & 2) << 1) | ((j & 4) >> 1)) : j; }

int zo_gate_build(const char *name, const double *p, int np, int *kind, zo_c64 *out) {
    int arity, npar;
    if (!zo_gate_lookup(name, &arity, &npar)) return 0;
    if (np != npar) return 0;
    const zo_c64 one = cx(1.0, 0.0), zero = cx(0.0, 0.0);
    const double sq = FRAC_1_SQRT_2_;
    zo_c64 tmp[4];
    if (!strcmp(name, "id") || !strcmp(name, "u0")) {
        *kind = 1; out[0] = one; out[1] = one;
    } else if (!strcmp(name, "x")) {
        *kind = 0; out[0] = zero; out[1] = one; out[2] = one; out[3] = zero;
    } else if (!strcmp(name, "y")) {
        *kind = 0; out[0] = zero; out[1] = cx(0.0, -1.0); out[2] = cx(0.0, 1.0); out[3] = zero;
    } else if (!strcmp(name, "z")) {
        *kind = 1; out[0] = one; out[1] = cx(-1.0, 0.0);
    } else if (!strcmp(name, "h")) {
        *kind = 0; out[0] = cx(sq, 0.0); out[1] = cx(sq, 0.0); out[2] = cx(sq, 0.0); out[3] = cx(-sq, 0.0);
    } else if (!strcmp(name, "s")) {
        *kind = 1; out[0] = one; out[1] = cx(0.0, 1.0);
    } else if (!strcmp(name, "sdg")) {
        *kind = 1; out[0] = one; out[1] = cx(0.0, -1.0);
    } else if (!strcmp(name, "t")) {
        *kind = 1; out[0] = one; out[1] = expi(FRAC_PI_4_);
    } else if (!strcmp(name, "tdg")) {
        *kind = 1; out[0] = one; out[1] = expi(-FRAC_PI_4_);
    } else if (!strcmp(name, "sx")) {
        *kind = 0; out[0] = cx(0.5, 0.5); out[1] = cx(0.5, -0.5); out[2] = cx(0.5, -0.5); out[3] = cx(0.5, 0.5);
    } else if (!strcmp(name, "sxdg")) {
        *kind = 0; out[0] = cx(0.5, -0.5); out[1] = cx(0.5, 0.5); out[2] = cx(0.5, 0.5); out[3] = cx(0.5, -0.5);
    } else if (!strcmp(name, "rx")) {
        *kind = 0; rxm(p[0], out);
    } else if (!strcmp(name, "ry")) {
        *kind = 0; rym(p[0], out);
    } else if (!strcmp(name, "rz")) {
        *kind = 1; rz_diag(p[0], out);
    } else if (!strcmp(name, "u1") || !strcmp(name, "p")) {
        *kind = 1; out[0] = one; out[1] = expi(p[0]);
    } else if (!strcmp(name, "u2")) {
        *kind = 0; u3m(FRAC_PI_2_, p[0], p[1], out);
    } else if (!strcmp(name, "u3") || !strcmp(name, "u")) {
        *kind = 0; u3m(p[0], p[1], p[2], out);
    } else if (!strcmp(name, "cx")) {
        *kind = 0; permutation(4, perm_cx, out);
    } else if (!strcmp(name, "cy")) {
        tmp[0] = zero; tmp[1] = cx(0.0, -1.0); tmp[2] = cx(0.0, 1.0); tmp[3] = zero;
        *kind = 0; controlled1(tmp, out);
    } else if (!strcmp(name, "cz")) {
        *kind = 1; out[0] = one; out[1] = one; out[2] = one; out[3] = cx(-1.0, 0.0);
    } else if (!strcmp(name, "ch")) {
        tmp[0] = cx(sq, 0.0); tmp[1] = cx(sq, 0.0); tmp[2] = cx(sq, 0.0); tmp[3] = cx(-sq, 0.0);
        *kind = 0; controlled1(tmp, out);
    } else if (!strcmp(name, "swap")) {
        *kind = 0; permutation(4, perm_swap, out);
    } else if (!strcmp(name, "cp") || !strcmp(name, "cu1")) {
        *kind = 1; out[0] = one; out[1] = one; out[2] = one; out[3] = expi(p[0]);
    } else if (!strcmp(name, "crx")) {
        rxm(p[0], tmp); *kind = 0; controlled1(tmp, out);
    } else if (!strcmp(name, "cry")) {
        rym(p[0], tmp); *kind = 0; controlled1(tmp, out);
    } else if (!strcmp(name, "crz")) {
        rz_diag(p[0], tmp);
        *kind = 1; out[0] = one; out[1] = tmp[0]; out[2] = one; out[3] = tmp[1];
    } else if (!strcmp(name, "cu3")) {
        u3m(p[0], p[1], p[2], tmp); *kind = 0; controlled1(tmp, out);
    } else if (!strcmp(name, "rxx")) {
        double ct = cos(p[0] / 2.0), st = sin(p[0] / 2.0);
        *kind = 0;
        for (int i = 0; i < 16; i++) out[i] = zero;
        for (int j = 0; j < 4; j++) {
            out[j * 4 + j] = cx(ct, 0.0);
            out[(j ^ 3) * 4 + j] = cx(0.0, -st);
        }
    } else if (!strcmp(name, "rzz")) {
        zo_c64 e0 = expi(-p[0] / 2.0), e1 = expi(p[0] / 2.0);
        *kind = 1; out[0] = e0; out[1] = e1; out[2] = e1; out[3] = e0;
    } else if (!strcmp(name, "ccx")) {
        *kind = 0; permutation(8, perm_ccx, out);
    } else if (!strcmp(name, "cswap")) {
        *kind = 0; permutation(8, perm_cswap, out);
    } else {
        return 0;
    }
    return arity;
}

/* ===================================================================== */
/* Compiler (src/compiler.rs:118-626).                                    */
/* ===================================================================== */

struct zo_compiled {
    uint32_t n_qubits, n_clbits;
    zo_op *ops;
    size_t nops;
    int dynamic;
    uint32_t *fq, *fc;
    size_t nfinal;
    zo_stats stats;
};

typedef struct {
    zo_op *v;
    size_t n, cap;
} opvec;

static void opvec_push(opvec *ov, zo_op op) {
    if (ov->n == ov->cap) {
        ov->cap = ov->cap ? ov->cap * 2 : 64;
        ov->v = (zo_op *)realloc(ov->v, ov->cap * sizeof(zo_op));
    }
    ov->v[ov->n++] = op;
}

static zo_op op_blank(int kind) {
    zo_op o;
    memset(&o, 0, sizeof(o));
    o.kind = kind;
    return o;
}

/* Gate-like op support (COp::gate_support, compiler.rs:57-63); If-wrapped
 * ops have none. Returns the support size or -1. CX support is
 * [control, target] in argument order. */
static int gate_support(const zo_op *o, uint32_t *sup) {
    if (o->has_if) return -1;
    if (o->kind == ZO_OP_UNITARY || o->kind == ZO_OP_DIAG) {
        for (uint32_t i = 0; i < o->k; i++) sup[i] = o->qubits[i];
        return (int)o->k;
    }
    if (o->kind == ZO_OP_CX) {
        sup[0] = o->control;
        sup[1] = o->target;
        return 2;
    }
    return -1;
}

static int is_self_inverse(const char *n) {
    static const char *si[] = {"x", "y", "z", "h", "cx", "cy", "cz", "ch", "swap", "ccx", "cswap"};
    for (size_t i = 0; i < sizeof(si) / sizeof(si[0]); i++)
        if (!strcmp(si[i], n)) return 1;
    return 0;
}

/* count_gates (compiler.rs:202-211): a Gate counts 1, an If counts its op. */
static size_t count_gates(const zo_instr *ins, size_t n) {
    size_t c = 0;
    for (size_t i = 0; i < n; i++)
        if (ins[i].kind == ZO_I_GATE) c++;
    return c;
}

/* cancel (compiler.rs:215-239). */
static zo_instr *cancel(const zo_instr *ins, size_t n, size_t *nout) {
    zo_instr *out = (zo_instr *)malloc((n ? n : 1) * sizeof(zo_instr));
    size_t m = 0;
    for (size_t x = 0; x < n; x++) {
        const zo_instr *g = &ins[x];
        int removed = 0;
        if (g->kind == ZO_I_GATE && g->cond_creg < 0 && g->np == 0 && is_self_inverse(g->name)) {
            for (size_t ii = m; ii-- > 0;) {
                const zo_instr *pg = &out[ii];
                if (pg->kind == ZO_I_GATE && pg->cond_creg < 0) {
                    int overlap = 0;
                    for (uint32_t a = 0; a < pg->nq; a++)
                        for (uint32_t b = 0; b < g->nq; b++)
                            if (pg->q[a] == g->q[b]) overlap = 1;
                    if (overlap) {
                        int same = !strcmp(pg->name, g->name) && pg->nq == g->nq;
                        for (uint32_t a = 0; same && a < g->nq; a++)
                            if (pg->q[a] != g->q[a]) same = 0;
                        if (same) {
                            memmove(&out[ii], &out[ii + 1], (m - ii - 1) * sizeof(zo_instr));
                            m--;
                            removed = 1;
                        }
                        break;
                    }
                } else {
                    break;
                }
            }
        }
        if (!removed) out[m++] = *g;
    }
    *nout = m;
    return out;
}

static void sort_u32(uint32_t *a, int n) {
    for (int i = 1; i < n; i++) {
        uint32_t v = a[i];
        int j = i - 1;
        while (j >= 0 && a[j] > v) {
            a[j + 1] = a[j];
            j--;
        }
        a[j + 1] = v;
    }
}

/* arg_index (compiler.rs:351-358) */
static size_t arg_index(size_t j_sorted, const int *pos, int k) {
    size_t j = 0;
    for (int b = 0; b < k; b++) j |= ((j_sorted >> pos[b]) & 1) << b;
    return j;
}

/* permute_unitary_to_sorted / permute_diag_to_sorted (compiler.rs:370-398).
 * Writes sorted qubits into `sorted` and returns a newly allocated matrix. */
static zo_c64 *permute_to_sorted(const uint32_t *qubits, int k, const zo_c64 *m, int diag, uint32_t *sorted) {
    int pos[ZO_MAXQ];
    for (int i = 0; i < k; i++) sorted[i] = qubits[i];
    sort_u32(sorted, k);
    int same = 1;
    for (int b = 0; b < k; b++) {
        for (int s = 0; s < k; s++)
            if (sorted[s] == qubits[b]) pos[b] = s;
        if (sorted[b] != qubits[b]) same = 0;
    }
    size_t dim = (size_t)1 << k;
    size_t len = diag ? dim : dim * dim;
    zo_c64 *out = (zo_c64 *)malloc(len * sizeof(zo_c64));
    if (same) {
        memcpy(out, m, len * sizeof(zo_c64));
        return out;
    }
    if (diag) {
        for (size_t j = 0; j < dim; j++) out[j] = m[arg_index(j, pos, k)];
    } else {
        for (size_t i = 0; i < dim; i++) {
            size_t ia = arg_index(i, pos, k);
            for (size_t j = 0; j < dim; j++) out[i * dim + j] = m[ia * dim + arg_index(j, pos, k)];
        }
    }
    return out;
}

static void set_err(char *err, size_t len, const char *msg) {
    if (err && len) snprintf(err, len, "%s", msg);
}

/* lower_gate (compiler.rs:296-347). Returns 0 ok (op may be "none" via
 * *emitted = 0), nonzero on error. */
static int lower_gate(const zo_instr *g, uint32_t nq, zo_op *op, int *emitted, char *err, size_t el) {
    int arity, npar;
    char buf[160];
    *emitted = 0;
    if (!zo_gate_lookup(g->name, &arity, &npar)) {
        snprintf(buf, sizeof buf, "invalid circuit: unknown gate '%s'", g->name);
        set_err(err, el, buf);
        return 1;
    }
    if ((int)g->nq != arity) {
        snprintf(buf, sizeof buf, "invalid circuit: gate '%s' expects %d qubit(s), got %u", g->name, arity, g->nq);
        set_err(err, el, buf);
        return 1;
    }
    for (uint32_t i = 0; i < g->nq; i++) {
        if (g->q[i] >= nq) {
            snprintf(buf, sizeof buf, "invalid circuit: qubit %u out of range (have %u)", g->q[i], nq);
            set_err(err, el, buf);
            return 1;
        }
    }
    for (uint32_t i = 0; i < g->nq; i++)
        for (uint32_t j = i + 1; j < g->nq; j++)
            if (g->q[i] == g->q[j]) {
                snprintf(buf, sizeof buf, "invalid circuit: gate '%s' applied to duplicate qubits", g->name);
                set_err(err, el, buf);
                return 1;
            }
    if (!strcmp(g->name, "id") || !strcmp(g->name, "u0")) return 0;
    if (!strcmp(g->name, "cx")) {
        *op = op_blank(ZO_OP_CX);
        op->control = g->q[0];
        op->target = g->q[1];
        *emitted = 1;
        return 0;
    }
    zo_c64 m[64];
    int kind;
    if (!zo_gate_build(g->name, g->p, (int)g->np, &kind, m)) {
        snprintf(buf, sizeof buf, "invalid circuit: gate '%s' expects %d parameter(s), got %u", g->name, npar, g->np);
        set_err(err, el, buf);
        return 1;
    }
    *op = op_blank(kind == 0 ? ZO_OP_UNITARY : ZO_OP_DIAG);
    op->k = (uint32_t)arity;
    op->data = permute_to_sorted(g->q, arity, m, kind == 1, op->qubits);
    *emitted = 1;
    return 0;
}

static int union_sorted(const uint32_t *a, int na, const uint32_t *b, int nb, uint32_t *u) {
    int n = 0;
    uint32_t tmp[2 * ZO_MAXQ + 4];
    for (int i = 0; i < na; i++) tmp[n++] = a[i];
    for (int i = 0; i < nb; i++) tmp[n++] = b[i];
    sort_u32(tmp, n);
    int m = 0;
    for (int i = 0; i < n; i++)
        if (m == 0 || u[m - 1] != tmp[i]) u[m++] = tmp[i];
    return m;
}

static int pos_in(uint32_t q, const uint32_t *to, int nto) {
    for (int i = 0; i < nto; i++)
        if (to[i] == q) return i;
    return -1;
}

/* subset_index (compiler.rs:411-418) */
static size_t subset_index(size_t i_to, const uint32_t *from, int nfrom, const uint32_t *to, int nto) {
    size_t j = 0;
    for (int b = 0; b < nfrom; b++) {
        int p = pos_in(from[b], to, nto);
        j |= ((i_to >> p) & 1) << b;
    }
    return j;
}

static int same_set(const uint32_t *a, int na, const uint32_t *b, int nb) {
    if (na != nb) return 0;
    for (int i = 0; i < na; i++)
        if (a[i] != b[i]) return 0;
    return 1;
}

/* embed_unitary (compiler.rs:421-447) */
static zo_c64 *embed_unitary(const zo_c64 *mat, const uint32_t *from, int nf, const uint32_t *to, int nt) {
    size_t dim_to = (size_t)1 << nt, dim_from = (size_t)1 << nf;
    zo_c64 *out = (zo_c64 *)malloc(dim_to * dim_to * sizeof(zo_c64));
    if (same_set(from, nf, to, nt)) {
        memcpy(out, mat, dim_to * dim_to * sizeof(zo_c64));
        return out;
    }
    size_t from_mask = 0;
    for (int i = 0; i < nf; i++) from_mask |= (size_t)1 << pos_in(from[i], to, nt);
    size_t rest_mask = (dim_to - 1) & ~from_mask;
    for (size_t i = 0; i < dim_to * dim_to; i++) out[i] = cx(0.0, 0.0);
    for (size_t i = 0; i < dim_to; i++) {
        size_t ifrom = subset_index(i, from, nf, to, nt);
        size_t irest = i & rest_mask;
        for (size_t j = 0; j < dim_to; j++) {
            if ((j & rest_mask) != irest) continue;
            size_t jfrom = subset_index(j, from, nf, to, nt);
            out[i * dim_to + j] = mat[ifrom * dim_from + jfrom];
        }
    }
    return out;
}

/* embed_diag (compiler.rs:449-455) */
static zo_c64 *embed_diag(const zo_c64 *d, const uint32_t *from, int nf, const uint32_t *to, int nt) {
    size_t dim_to = (size_t)1 << nt;
    zo_c64 *out = (zo_c64 *)malloc(dim_to * sizeof(zo_c64));
    if (same_set(from, nf, to, nt)) {
        memcpy(out, d, dim_to * sizeof(zo_c64));
        return out;
    }
    for (size_t i = 0; i < dim_to; i++) out[i] = d[subset_index(i, from, nf, to, nt)];
    return out;
}

/* matmul (compiler.rs:457-471): out = a·b, loop order i, l, j, zero a-entries skipped. */
static zo_c64 *matmul(const zo_c64 *a, const zo_c64 *b, size_t dim) {
    zo_c64 *out = (zo_c64 *)calloc(dim * dim, sizeof(zo_c64));
    for (size_t i = 0; i < dim; i++)
        for (size_t l = 0; l < dim; l++) {
            zo_c64 ail = a[i * dim + l];
            if (ciszero(ail)) continue;
            for (size_t j = 0; j < dim; j++) out[i * dim + j] = cadd(out[i * dim + j], cmul(ail, b[l * dim + j]));
        }
    return out;
}

/* fuse_diagonals (compiler.rs:477-535) */
static opvec fuse_diagonals(opvec in, int diag_max) {
    opvec out = {0};
    int have = 0;
    zo_op cur;
    uint64_t blocked = 0;
    for (size_t x = 0; x < in.n; x++) {
        zo_op op = in.v[x];
        if (op.kind == ZO_OP_DIAG && !op.has_if) {
            int clean = 1;
            for (uint32_t i = 0; i < op.k; i++)
                if (blocked >> op.qubits[i] & 1) clean = 0;
            uint32_t u[2 * ZO_MAXQ];
            int nu = have ? union_sorted(cur.qubits, (int)cur.k, op.qubits, (int)op.k, u) : 0;
            if (have && clean && nu <= diag_max) {
                zo_c64 *a = embed_diag(cur.data, cur.qubits, (int)cur.k, u, nu);
                zo_c64 *b = embed_diag(op.data, op.qubits, (int)op.k, u, nu);
                size_t dim = (size_t)1 << nu;
                zo_c64 *t = (zo_c64 *)malloc(dim * sizeof(zo_c64));
                for (size_t i = 0; i < dim; i++) t[i] = cmul(a[i], b[i]);
                free(a);
                free(b);
                free(cur.data);
                free(op.data);
                cur.data = t;
                cur.k = (uint32_t)nu;
                memcpy(cur.qubits, u, nu * sizeof(uint32_t));
            } else {
                if (have) opvec_push(&out, cur);
                blocked = 0;
                cur = op;
                have = 1;
            }
        } else if ((op.kind == ZO_OP_UNITARY || op.kind == ZO_OP_CX) && !op.has_if) {
            uint32_t sup[ZO_MAXQ];
            int ns = gate_support(&op, sup);
            if (have) {
                int overlap = 0;
                for (int i = 0; i < ns; i++)
                    if (pos_in(sup[i], cur.qubits, (int)cur.k) >= 0) overlap = 1;
                if (overlap) {
                    opvec_push(&out, cur);
                    have = 0;
                    blocked = 0;
                } else {
                    for (int i = 0; i < ns; i++) blocked |= (uint64_t)1 << sup[i];
                }
            }
            opvec_push(&out, op);
        } else {
            if (have) opvec_push(&out, cur);
            have = 0;
            blocked = 0;
            opvec_push(&out, op);
        }
    }
    if (have) opvec_push(&out, cur);
    free(in.v);
    return out;
}

static const zo_c64 *cx_matrix(void) {
    static zo_c64 m[16];
    static int init = 0;
    if (!init) {
        permutation(4, perm_cx, m);
        init = 1;
    }
    return m;
}

/* to_matrix inside fuse_general (compiler.rs:550-571). */
static zo_c64 *to_matrix(const zo_op *op, uint32_t *sup, int *k) {
    if (op->kind == ZO_OP_UNITARY) {
        size_t dim = (size_t)1 << op->k;
        zo_c64 *m = (zo_c64 *)malloc(dim * dim * sizeof(zo_c64));
        memcpy(m, op->data, dim * dim * sizeof(zo_c64));
        memcpy(sup, op->qubits, op->k * sizeof(uint32_t));
        *k = (int)op->k;
        return m;
    }
    if (op->kind == ZO_OP_DIAG) {
        size_t dim = (size_t)1 << op->k;
        zo_c64 *m = (zo_c64 *)calloc(dim * dim, sizeof(zo_c64));
        for (size_t j = 0; j < dim; j++) m[j * dim + j] = op->data[j];
        memcpy(sup, op->qubits, op->k * sizeof(uint32_t));
        *k = (int)op->k;
        return m;
    }
    /* CX */
    uint32_t q[2] = {op->control, op->target};
    *k = 2;
    return permute_to_sorted(q, 2, cx_matrix(), 0, sup);
}

/* fuse_general (compiler.rs:540-626) */
static opvec fuse_general(opvec in, int kmax) {
    opvec out = {0};
    int have = 0;
    uint32_t gsup[ZO_MAXQ];
    int gk = 0;
    zo_c64 *gmat = NULL;
    size_t gcount = 0;
    zo_op gfirst;
#define FLUSH()                                      \
    do {                                             \
        if (have) {                                  \
            if (gcount == 1) {                       \
                opvec_push(&out, gfirst);            \
                free(gmat);                          \
            } else {                                 \
                zo_op f = op_blank(ZO_OP_UNITARY);   \
                f.k = (uint32_t)gk;                  \
                memcpy(f.qubits, gsup, gk * 4);      \
                f.data = gmat;                       \
                opvec_push(&out, f);                 \
                free(gfirst.data);                   \
            }                                        \
            have = 0;                                \
            gmat = NULL;                             \
        }                                            \
    } while (0)
    for (size_t x = 0; x < in.n; x++) {
        zo_op op = in.v[x];
        uint32_t sup[ZO_MAXQ];
        int ns = gate_support(&op, sup);
        int fusable = ns >= 0 && ns <= kmax;
        if (!fusable) {
            FLUSH();
            opvec_push(&out, op);
            continue;
        }
        if (!have) {
            gmat = to_matrix(&op, gsup, &gk);
            gcount = 1;
            gfirst = op;
            have = 1;
            continue;
        }
        uint32_t qs[ZO_MAXQ];
        int k;
        zo_c64 *m = to_matrix(&op, qs, &k);
        uint32_t u[2 * ZO_MAXQ];
        int nu = union_sorted(gsup, gk, qs, k, u);
        if (nu <= kmax) {
            zo_c64 *cur_e = embed_unitary(gmat, gsup, gk, u, nu);
            zo_c64 *op_e = embed_unitary(m, qs, k, u, nu);
            zo_c64 *prod = matmul(op_e, cur_e, (size_t)1 << nu);
            free(cur_e);
            free(op_e);
            free(m);
            free(gmat);
            gmat = prod;
            gk = nu;
            memcpy(gsup, u, nu * 4);
            gcount++;
            free(op.data);
        } else {
            free(m);
            FLUSH();
            gmat = to_matrix(&op, gsup, &gk);
            gcount = 1;
            gfirst = op;
            have = 1;
        }
    }
    FLUSH();
#undef FLUSH
    free(in.v);
    return out;
}

int zo_compile(uint32_t n_qubits, const uint32_t *creg_sizes, uint32_t n_cregs, const zo_instr *ins, size_t n_ins,
               uint32_t fusion_max, uint32_t diag_max, zo_compiled **outp, char *err, size_t el) {
    char buf[200];
    uint32_t n_clbits = 0;
    for (uint32_t i = 0; i < n_cregs; i++) n_clbits += creg_sizes[i];
    if (n_qubits == 0) {
        set_err(err, el, "invalid circuit: no qubits declared");
        return 1;
    }
    if (n_qubits > 48) {
        snprintf(buf, sizeof buf, "invalid circuit: %u qubits is beyond any state-vector budget", n_qubits);
        set_err(err, el, buf);
        return 1;
    }
    if (n_clbits > 64) {
        set_err(err, el, "invalid circuit: more than 64 classical bits are not supported");
        return 1;
    }
    size_t input_gates = count_gates(ins, n_ins);
    size_t nc;
    zo_instr *cin = cancel(ins, n_ins, &nc);
    size_t cancelled = input_gates - count_gates(cin, nc);

    opvec ops = {0};
    for (size_t x = 0; x < nc; x++) {
        const zo_instr *g = &cin[x];
        zo_op op;
        int emitted = 0;
        if (g->kind == ZO_I_GATE) {
            if (lower_gate(g, n_qubits, &op, &emitted, err, el)) goto fail;
        } else if (g->kind == ZO_I_MEASURE || g->kind == ZO_I_RESET) {
            uint32_t q = g->q[0];
            if (q >= n_qubits) {
                snprintf(buf, sizeof buf, "invalid circuit: qubit %u out of range (have %u)", q, n_qubits);
                set_err(err, el, buf);
                goto fail;
            }
            if (g->kind == ZO_I_MEASURE) {
                if (g->clbit >= n_clbits) {
                    snprintf(buf, sizeof buf, "invalid circuit: clbit %u out of range (have %u)", g->clbit, n_clbits);
                    set_err(err, el, buf);
                    goto fail;
                }
                op = op_blank(ZO_OP_MEASURE);
                op.qubit = q;
                op.clbit = g->clbit;
            } else {
                op = op_blank(ZO_OP_RESET);
                op.qubit = q;
            }
            emitted = 1;
        } else {
            op = op_blank(ZO_OP_BARRIER);
            emitted = 1;
        }
        if (emitted && g->cond_creg >= 0) {
            if ((uint32_t)g->cond_creg >= n_cregs) {
                snprintf(buf, sizeof buf, "invalid circuit: creg #%d out of range", g->cond_creg);
                set_err(err, el, buf);
                free(op.data);
                goto fail;
            }
            uint32_t off = 0;
            for (int i = 0; i < g->cond_creg; i++) off += creg_sizes[i];
            op.has_if = 1;
            op.creg_offset = off;
            op.creg_len = creg_sizes[g->cond_creg];
            op.value = g->cond_value;
        }
        if (emitted) opvec_push(&ops, op);
    }
    free(cin);
    cin = NULL;

    if (fusion_max > 6) fusion_max = 6;
    if (diag_max > 12) diag_max = 12;
    if (fusion_max >= 1) {
        ops = fuse_diagonals(ops, (int)diag_max);
        ops = fuse_general(ops, (int)fusion_max);
    }
    /* strip barriers */
    {
        size_t m = 0;
        for (size_t i = 0; i < ops.n; i++)
            if (!(ops.v[i].kind == ZO_OP_BARRIER && !ops.v[i].has_if)) ops.v[m++] = ops.v[i];
        ops.n = m;
    }
    zo_compiled *c = (zo_compiled *)calloc(1, sizeof(zo_compiled));
    c->n_qubits = n_qubits;
    c->n_clbits = n_clbits;
    size_t split = ops.n;
    while (split > 0 && ops.v[split - 1].kind == ZO_OP_MEASURE && !ops.v[split - 1].has_if) split--;
    int body_dynamic = 0;
    for (size_t i = 0; i < split; i++) {
        const zo_op *o = &ops.v[i];
        if (o->has_if || o->kind == ZO_OP_MEASURE || o->kind == ZO_OP_RESET) body_dynamic = 1;
    }
    if (body_dynamic) {
        c->dynamic = 1;
    } else {
        c->nfinal = ops.n - split;
        c->fq = (uint32_t *)malloc((c->nfinal + 1) * 4);
        c->fc = (uint32_t *)malloc((c->nfinal + 1) * 4);
        for (size_t i = 0; i < c->nfinal; i++) {
            c->fq[i] = ops.v[split + i].qubit;
            c->fc[i] = ops.v[split + i].clbit;
        }
        ops.n = split;
    }
    c->ops = ops.v;
    c->nops = ops.n;
    size_t maxf = 0;
    for (size_t i = 0; i < ops.n; i++) {
        uint32_t sup[ZO_MAXQ];
        int ns = gate_support(&ops.v[i], sup);
        if (ns > 0 && (size_t)ns > maxf) maxf = (size_t)ns;
    }
    c->stats.input_gates = input_gates;
    c->stats.cancelled = cancelled;
    c->stats.output_ops = ops.n;
    c->stats.max_fused = maxf;
    *outp = c;
    return 0;
fail:
    free(cin);
    for (size_t i = 0; i < ops.n; i++) free(ops.v[i].data);
    free(ops.v);
    return 1;
}

void zo_compiled_free(zo_compiled *c) {
    if (!c) return;
    for (size_t i = 0; i < c->nops; i++) free(c->ops[i].data);
    free(c->ops);
    free(c->fq);
    free(c->fc);
    free(c);
}
size_t zo_compiled_nops(const zo_compiled *c) { return c->nops; }
const zo_op *zo_compiled_op(const zo_compiled *c, size_t i) { return &c->ops[i]; }
int zo_compiled_dynamic(const zo_compiled *c) { return c->dynamic; }
size_t zo_compiled_nfinal(const zo_compiled *c) { return c->nfinal; }
void zo_compiled_final(const zo_compiled *c, size_t i, uint32_t *q, uint32_t *cb) {
    *q = c->fq[i];
    *cb = c->fc[i];
}
void zo_compiled_stats(const zo_compiled *c, zo_stats *s) { *s = c->stats; }

/* ===================================================================== */
/* CPU backend: scalar kernels of src/state.rs with the same trees.       */
/* ===================================================================== */

struct zo_state {
    uint32_t n;
    int prec; /* 32 or 64 */
    void *re, *im;
};

static int g_threads = 0;
void zo_set_threads(int t) {
    g_threads = t;
    omp_set_num_threads(t > 0 ? t : omp_get_num_procs());
}
int zo_get_threads(void) { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

/* Work split: like task_ranges (state.rs:90-105) — at most 8x threads
 * tasks of at least 2^13 items; below that a single task. Only the
 * elementwise kernels use it, so the split never changes results. */
#define PAR_MIN ((size_t)1 << 13)
static size_t ntasks_for(size_t total) {
    if (total <= PAR_MIN) return 1;
    size_t t = total / PAR_MIN, cap = (size_t)zo_get_threads() * 8;
    if (t > cap) t = cap;
    return t ? t : 1;
}

/* insert_zeros (state.rs:162-169) */
static inline size_t insert_zeros(size_t g, const uint32_t *qs, int k) {
    size_t x = g;
    for (int i = 0; i < k; i++) {
        uint32_t q = qs[i];
        size_t low = x & (((size_t)1 << q) - 1);
        x = ((x >> q) << (q + 1)) | low;
    }
    return x;
}

#define DEFINE_KERNELS(T, S)                                                                          \
    /* kern_1q_scalar (state.rs:232-260) */                                                            \
    static void k1q_##S(T *re, T *im, uint32_t q, size_t h0, size_t h1, const T *m) {                  \
        size_t s = (size_t)1 << q, mask = s - 1;                                                       \
        T m00r = m[0], m00i = m[1], m01r = m[2], m01i = m[3], m10r = m[4], m10i = m[5], m11r = m[6],   \
          m11i = m[7];                                                                                 \
        for (size_t h = h0; h < h1; h++) {                                                             \
            size_t a = ((h >> q) << (q + 1)) | (h & mask), b = a + s;                                  \
            T ar = re[a], ai = im[a], br = re[b], bi = im[b];                                          \
            re[a] = m00r * ar - m00i * ai + m01r * br - m01i * bi;                                     \
            im[a] = m00r * ai + m00i * ar + m01r * bi + m01i * br;                                     \
            re[b] = m10r * ar - m10i * ai + m11r * br - m11i * bi;                                     \
            im[b] = m10r * ai + m10i * ar + m11r * bi + m11i * br;                                     \
        }                                                                                              \
    }                                                                                                  \
    static void apply_1q_##S(zo_state *st, uint32_t q, const zo_c64 *mc) {                             \
        T m[8];                                                                                        \
        for (int i = 0; i < 4; i++) {                                                                  \
            m[2 * i] = (T)mc[i].re;                                                                    \
            m[2 * i + 1] = (T)mc[i].im;                                                                \
        }                                                                                              \
        size_t half = ((size_t)1 << st->n) >> 1, nt = ntasks_for(half), per = (half + nt - 1) / nt;    \
        T *re = (T *)st->re, *im = (T *)st->im;                                                        \
        _Pragma("omp parallel for schedule(static)") for (size_t t = 0; t < nt; t++) {                 \
            size_t h0 = t * per, h1 = (t + 1) * per < half ? (t + 1) * per : half;                     \
            if (h0 < h1) k1q_##S(re, im, q, h0, h1, m);                                                \
        }                                                                                              \
    }                                                                                                  \
    /* kern_kq_scalar (state.rs:355-392) */                                                            \
    static void apply_kq_##S(zo_state *st, const uint32_t *qs, uint32_t k, const zo_c64 *mc) {        \
        size_t dim = (size_t)1 << k;                                                                   \
        T *mre = (T *)malloc(dim * dim * sizeof(T)), *mim = (T *)malloc(dim * dim * sizeof(T));        \
        for (size_t i = 0; i < dim * dim; i++) {                                                       \
            mre[i] = (T)mc[i].re;                                                                      \
            mim[i] = (T)mc[i].im;                                                                      \
        }                                                                                              \
        size_t offs[1 << 7];                                                                           \
        for (size_t j = 0; j < dim; j++) {                                                             \
            size_t o = 0;                                                                              \
            for (uint32_t b = 0; b < k; b++)                                                           \
                if ((j >> b) & 1) o |= (size_t)1 << qs[b];                                             \
            offs[j] = o;                                                                               \
        }                                                                                              \
        size_t groups = ((size_t)1 << st->n) >> k, nt = ntasks_for(groups),                            \
               per = (groups + nt - 1) / nt;                                                           \
        T *re = (T *)st->re, *im = (T *)st->im;                                                        \
        _Pragma("omp parallel for schedule(static)") for (size_t t = 0; t < nt; t++) {                 \
            T xr[128], xi[128], yr[128], yi[128];                                                      \
            size_t g0 = t * per, g1 = (t + 1) * per < groups ? (t + 1) * per : groups;                 \
            for (size_t g = g0; g < g1; g++) {                                                         \
                size_t base = insert_zeros(g, qs, (int)k);                                             \
                for (size_t j = 0; j < dim; j++) {                                                     \
                    xr[j] = re[base | offs[j]];                                                        \
                    xi[j] = im[base | offs[j]];                                                        \
                }                                                                                      \
                for (size_t r = 0; r < dim; r++) {                                                     \
                    T ar = (T)0, ai = (T)0;                                                            \
                    for (size_t c = 0; c < dim; c++) {                                                 \
                        T wr = mre[r * dim + c], wi = mim[r * dim + c];                                \
                        ar = ar + wr * xr[c] - wi * xi[c];                                             \
                        ai = ai + wr * xi[c] + wi * xr[c];                                             \
                    }                                                                                  \
                    yr[r] = ar;                                                                        \
                    yi[r] = ai;                                                                        \
                }                                                                                      \
                for (size_t j = 0; j < dim; j++) {                                                     \
                    re[base | offs[j]] = yr[j];                                                        \
                    im[base | offs[j]] = yi[j];                                                        \
                }                                                                                      \
            }                                                                                          \
        }                                                                                              \
        free(mre);                                                                                     \
        free(mim);                                                                                     \
    }                                                                                                  \
    /* apply_cx (state.rs:397-417) */                                                                  \
    static void apply_cx_##S(zo_state *st, uint32_t c, uint32_t tq) {                                 \
        uint32_t qs[2] = {c < tq ? c : tq, c < tq ? tq : c};                                           \
        size_t coff = (size_t)1 << c, toff = (size_t)1 << tq;                                          \
        size_t groups = ((size_t)1 << st->n) >> 2, nt = ntasks_for(groups),                            \
               per = (groups + nt - 1) / nt;                                                           \
        T *re = (T *)st->re, *im = (T *)st->im;                                                        \
        _Pragma("omp parallel for schedule(static)") for (size_t t = 0; t < nt; t++) {                 \
            size_t g0 = t * per, g1 = (t + 1) * per < groups ? (t + 1) * per : groups;                 \
            for (size_t g = g0; g < g1; g++) {                                                         \
                size_t a = insert_zeros(g, qs, 2) | coff, b = a | toff;                                \
                T x = re[a];                                                                           \
                re[a] = re[b];                                                                         \
                re[b] = x;                                                                             \
                x = im[a];                                                                             \
                im[a] = im[b];                                                                         \
                im[b] = x;                                                                             \
            }                                                                                          \
        }                                                                                              \
    }                                                                                                  \
    /* apply_diag: kern_diag1_scalar (state.rs:498-527), kern_diagk_scalar (:577-596) */               \
    static void apply_diag_##S(zo_state *st, const uint32_t *qs, uint32_t k, const zo_c64 *d) {       \
        T *re = (T *)st->re, *im = (T *)st->im;                                                        \
        if (k == 1) {                                                                                  \
            uint32_t q = qs[0];                                                                        \
            T d0r = (T)d[0].re, d0i = (T)d[0].im, d1r = (T)d[1].re, d1i = (T)d[1].im;                  \
            size_t half = ((size_t)1 << st->n) >> 1, nt = ntasks_for(half), per = (half + nt - 1) / nt; \
            size_t s = (size_t)1 << q, mask = s - 1;                                                   \
            _Pragma("omp parallel for schedule(static)") for (size_t t = 0; t < nt; t++) {             \
                size_t h0 = t * per, h1 = (t + 1) * per < half ? (t + 1) * per : half;                 \
                for (size_t h = h0; h < h1; h++) {                                                     \
                    size_t a = ((h >> q) << (q + 1)) | (h & mask), b = a + s;                          \
                    T ar = re[a], ai = im[a];                                                          \
                    re[a] = d0r * ar - d0i * ai;                                                       \
                    im[a] = d0r * ai + d0i * ar;                                                       \
                    T br = re[b], bi = im[b];                                                          \
                    re[b] = d1r * br - d1i * bi;                                                       \
                    im[b] = d1r * bi + d1i * br;                                                       \
                }                                                                                      \
            }                                                                                          \
            return;                                                                                    \
        }                                                                                              \
        size_t dim = (size_t)1 << k;                                                                   \
        T *dre = (T *)malloc(dim * sizeof(T)), *dim_ = (T *)malloc(dim * sizeof(T));                   \
        for (size_t j = 0; j < dim; j++) {                                                             \
            dre[j] = (T)d[j].re;                                                                       \
            dim_[j] = (T)d[j].im;                                                                      \
        }                                                                                              \
        size_t len = (size_t)1 << st->n, nt = ntasks_for(len), per = (len + nt - 1) / nt;              \
        _Pragma("omp parallel for schedule(static)") for (size_t t = 0; t < nt; t++) {                 \
            size_t i0 = t * per, i1 = (t + 1) * per < len ? (t + 1) * per : len;                       \
            for (size_t i = i0; i < i1; i++) {                                                         \
                size_t j = 0;                                                                          \
                for (uint32_t b = 0; b < k; b++) j |= ((i >> qs[b]) & 1) << b;                         \
                T wr = dre[j], wi = dim_[j], ar = re[i], ai = im[i];                                   \
                re[i] = wr * ar - wi * ai;                                                             \
                im[i] = wr * ai + wi * ar;                                                             \
            }                                                                                          \
        }                                                                                              \
        free(dre);                                                                                     \
        free(dim_);                                                                                    \
    }                                                                                                  \
    /* prob_one (state.rs:599-626): f64 accumulation of |amp|^2 over the q=1 half. Fixed order:       \
     * serial within 2^16-half-index chunks, chunk partials summed in chunk order. */                  \
    static double prob_one_##S(zo_state *st, uint32_t q) {                                             \
        size_t half = ((size_t)1 << st->n) >> 1, s = (size_t)1 << q, mask = s - 1;                     \
        size_t ch = (size_t)1 << 16;                                                                   \
        if (ch > half) ch = half;                                                                      \
        size_t nch = (half + ch - 1) / ch;                                                             \
        double *part = (double *)malloc(nch * sizeof(double));                                         \
        const T *re = (const T *)st->re, *im = (const T *)st->im;                                      \
        _Pragma("omp parallel for schedule(static)") for (size_t c = 0; c < nch; c++) {                \
            size_t h0 = c * ch, h1 = h0 + ch < half ? h0 + ch : half;                                  \
            double acc = 0.0;                                                                          \
            for (size_t h = h0; h < h1; h++) {                                                         \
                size_t b = (((h >> q) << (q + 1)) | (h & mask)) + s;                                   \
                double r = (double)re[b], i = (double)im[b];                                           \
                acc += r * r + i * i;                                                                  \
            }                                                                                          \
            part[c] = acc;                                                                             \
        }                                                                                              \
        double tot = 0.0;                                                                              \
        for (size_t c = 0; c < nch; c++) tot += part[c];                                               \
        free(part);                                                                                    \
        return tot;                                                                                    \
    }                                                                                                  \
    /* collapse (state.rs:630-661) */                                                                  \
    static void collapse_##S(zo_state *st, uint32_t q, int outcome, double prob) {                     \
        T scale = (T)(1.0 / sqrt(prob));                                                               \
        size_t half = ((size_t)1 << st->n) >> 1, s = (size_t)1 << q, mask = s - 1;                     \
        size_t nt = ntasks_for(half), per = (half + nt - 1) / nt;                                      \
        T *re = (T *)st->re, *im = (T *)st->im;                                                        \
        _Pragma("omp parallel for schedule(static)") for (size_t t = 0; t < nt; t++) {                 \
            size_t h0 = t * per, h1 = (t + 1) * per < half ? (t + 1) * per : half;                     \
            for (size_t h = h0; h < h1; h++) {                                                         \
                size_t a0 = ((h >> q) << (q + 1)) | (h & mask);                                        \
                size_t keep = outcome ? a0 + s : a0, zero = outcome ? a0 : a0 + s;                     \
                re[keep] = re[keep] * scale;                                                           \
                im[keep] = im[keep] * scale;                                                           \
                re[zero] = (T)0;                                                                       \
                im[zero] = (T)0;                                                                       \
            }                                                                                          \
        }                                                                                              \
    }                                                                                                  \
    /* norm_sqr (state.rs:143-156): serial per 2^16 chunk, partials summed in order. */               \
    static double norm_##S(zo_state *st) {                                                             \
        size_t len = (size_t)1 << st->n, ch = (size_t)1 << 16;                                         \
        if (ch > len) ch = len;                                                                        \
        size_t nch = (len + ch - 1) / ch;                                                              \
        double *part = (double *)malloc(nch * sizeof(double));                                         \
        const T *re = (const T *)st->re, *im = (const T *)st->im;                                      \
        _Pragma("omp parallel for schedule(static)") for (size_t c = 0; c < nch; c++) {                \
            size_t i0 = c * ch, i1 = i0 + ch < len ? i0 + ch : len;                                    \
            double acc = 0.0;                                                                          \
            for (size_t i = i0; i < i1; i++) {                                                         \
                double r = (double)re[i], x = (double)im[i];                                           \
                acc += r * r + x * x;                                                                  \
            }                                                                                          \
            part[c] = acc;                                                                             \
        }                                                                                              \
        double tot = 0.0;                                                                              \
        for (size_t c = 0; c < nch; c++) tot += part[c];                                               \
        free(part);                                                                                    \
        return tot;                                                                                    \
    }                                                                                                  \
    static inline double p2_##S(const zo_state *st, size_t i) {                                        \
        double r = (double)((const T *)st->re)[i], x = (double)((const T *)st->im)[i];                 \
        return r * r + x * x;                                                                          \
    }

DEFINE_KERNELS(double, f64)
DEFINE_KERNELS(float, f32)

zo_state *zo_state_new(uint32_t n, int prec) {
    zo_state *s = (zo_state *)calloc(1, sizeof(zo_state));
    s->n = n;
    s->prec = prec;
    size_t len = (size_t)1 << n, es = prec == 32 ? 4 : 8;
    s->re = calloc(len, es);
    s->im = calloc(len, es);
    if (!s->re || !s->im) {
        free(s->re);
        free(s->im);
        free(s);
        return NULL;
    }
    if (prec == 32)
        ((float *)s->re)[0] = 1.0f;
    else
        ((double *)s->re)[0] = 1.0;
    return s;
}

void zo_state_free(zo_state *s) {
    if (!s) return;
    free(s->re);
    free(s->im);
    free(s);
}

void zo_apply_unitary(zo_state *s, const uint32_t *qs, uint32_t k, const zo_c64 *m) {
    if (k == 1) {
        if (s->prec == 32) apply_1q_f32(s, qs[0], m);
        else apply_1q_f64(s, qs[0], m);
    } else {
        if (s->prec == 32) apply_kq_f32(s, qs, k, m);
        else apply_kq_f64(s, qs, k, m);
    }
}
void zo_apply_diagonal(zo_state *s, const uint32_t *qs, uint32_t k, const zo_c64 *d) {
    if (s->prec == 32) apply_diag_f32(s, qs, k, d);
    else apply_diag_f64(s, qs, k, d);
}
void zo_apply_cx(zo_state *s, uint32_t c, uint32_t t) {
    if (s->prec == 32) apply_cx_f32(s, c, t);
    else apply_cx_f64(s, c, t);
}
double zo_prob_one(zo_state *s, uint32_t q) { return s->prec == 32 ? prob_one_f32(s, q) : prob_one_f64(s, q); }

/* CpuBackend::measure (exec.rs:201-207) */
int zo_measure(zo_state *s, uint32_t q, double u) {
    double p1 = zo_prob_one(s, q);
    int outcome = u < p1;
    double p = outcome ? p1 : 1.0 - p1;
    if (s->prec == 32) collapse_f32(s, q, outcome, p);
    else collapse_f64(s, q, outcome, p);
    return outcome;
}

/* StateVec::reset_zero (state.rs:128-132) */
void zo_reset_all(zo_state *s) {
    size_t len = (size_t)1 << s->n, es = s->prec == 32 ? 4 : 8;
    memset(s->re, 0, len * es);
    memset(s->im, 0, len * es);
    if (s->prec == 32) ((float *)s->re)[0] = 1.0f;
    else ((double *)s->re)[0] = 1.0;
}

double zo_norm_sqr(zo_state *s) { return s->prec == 32 ? norm_f32(s) : norm_f64(s); }

void zo_statevector(zo_state *s, zo_c64 *out) {
    size_t len = (size_t)1 << s->n;
    for (size_t i = 0; i < len; i++) {
        if (s->prec == 32) out[i] = cx((double)((float *)s->re)[i], (double)((float *)s->im)[i]);
        else out[i] = cx(((double *)s->re)[i], ((double *)s->im)[i]);
    }
}

void zo_load_state(zo_state *s, const zo_c64 *in) {
    size_t len = (size_t)1 << s->n;
    for (size_t i = 0; i < len; i++) {
        if (s->prec == 32) {
            ((float *)s->re)[i] = (float)in[i].re;
            ((float *)s->im)[i] = (float)in[i].im;
        } else {
            ((double *)s->re)[i] = in[i].re;
            ((double *)s->im)[i] = in[i].im;
        }
    }
}

static double p2(const zo_state *s, size_t i) { return s->prec == 32 ? p2_f32(s, i) : p2_f64(s, i); }

static int cmp_f64(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* sample_indices (sample.rs:29-111) with Xoshiro256++::seed_from_u64(seed)
 * (CpuBackend::sample, exec.rs:213-216). Output ascending. */
void zo_sample(zo_state *s, uint64_t shots, uint64_t seed, uint64_t *out) {
    if (shots == 0) return;
    zo_rng rng;
    zo_rng_seed(&rng, seed);
    size_t n = (size_t)1 << s->n, chunk = n < ((size_t)1 << 16) ? n : ((size_t)1 << 16);
    size_t nch = (n + chunk - 1) / chunk;
    double *sums = (double *)malloc(nch * sizeof(double));
#pragma omp parallel for schedule(static)
    for (size_t c = 0; c < nch; c++) {
        size_t lo = c * chunk, hi = lo + chunk < n ? lo + chunk : n;
        double acc = 0.0;
        for (size_t i = lo; i < hi; i++) acc += p2(s, i);
        sums[c] = acc;
    }
    double *cum = (double *)malloc((nch + 1) * sizeof(double));
    cum[0] = 0.0;
    for (size_t c = 0; c < nch; c++) cum[c + 1] = cum[c] + sums[c];
    double total = cum[nch];
    double *us = (double *)malloc(shots * sizeof(double));
    for (uint64_t i = 0; i < shots; i++) us[i] = zo_rng_f64(&rng) * total;
    qsort(us, shots, sizeof(double), cmp_f64);
    size_t *starts = (size_t *)malloc((nch + 1) * sizeof(size_t));
    for (size_t c = 0; c <= nch; c++) {
        /* partition_point(|u| u < cum[c]) */
        size_t lo = 0, hi = shots;
        while (lo < hi) {
            size_t mid = lo + (hi - lo) / 2;
            if (us[mid] < cum[c]) lo = mid + 1;
            else hi = mid;
        }
        starts[c] = lo;
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (size_t c = 0; c < nch; c++) {
        if (!(starts[c] < starts[c + 1])) continue;
        size_t lo = c * chunk, hi = lo + chunk < n ? lo + chunk : n;
        size_t s0 = starts[c], s1 = starts[c + 1], ptr = s0;
        double acc = cum[c];
        for (size_t i = lo; i < hi; i++) {
            acc += p2(s, i);
            while (ptr < s1 && us[ptr] < acc) out[ptr++] = (uint64_t)i;
            if (ptr == s1) break;
        }
        if (ptr < s1) {
            size_t last_nz = hi - 1;
            for (size_t i = hi; i-- > lo;) {
                if (p2(s, i) > 0.0) {
                    last_nz = i;
                    break;
                }
            }
            while (ptr < s1) out[ptr++] = (uint64_t)last_nz;
        }
    }
    free(sums);
    free(cum);
    free(us);
    free(starts);
}

/* ===================================================================== */
/* Noise (src/noise.rs:91-192).                                           */
/* ===================================================================== */

static void apply_pauli(zo_state *s, uint32_t q, uint64_t code) {
    zo_c64 one = cx(1.0, 0.0), zero = cx(0.0, 0.0);
    if (code == 1) {
        zo_c64 m[4] = {zero, one, one, zero};
        zo_apply_unitary(s, &q, 1, m);
    } else if (code == 2) {
        zo_c64 m[4] = {zero, cx(0.0, -1.0), cx(0.0, 1.0), zero};
        zo_apply_unitary(s, &q, 1, m);
    } else if (code == 3) {
        zo_c64 d[2] = {one, cx(-1.0, 0.0)};
        zo_apply_diagonal(s, &q, 1, d);
    }
}

static void amplitude_damp(zo_state *s, uint32_t q, double gamma, double u) {
    double p_jump = gamma * zo_prob_one(s, q);
    if (u < p_jump) {
        zo_measure(s, q, 0.0);
        apply_pauli(s, q, 1);
    } else {
        double sc = 1.0 / sqrt(1.0 - p_jump);
        zo_c64 d[2] = {cx(sc, 0.0), cx(sc * sqrt(1.0 - gamma), 0.0)};
        zo_apply_diagonal(s, &q, 1, d);
    }
}

static void apply_gate_noise(zo_state *s, const zo_noise *m, const uint32_t *qs, uint32_t k, zo_rng *rng) {
    double p_dep = k == 1 ? m->depolarizing_1q : m->depolarizing_2q;
    if (p_dep > 0.0 && zo_rng_f64(rng) < p_dep) {
        uint64_t idx = zo_rng_range(rng, 1, (uint64_t)1 << (2 * k));
        for (uint32_t b = 0; b < k; b++) apply_pauli(s, qs[b], (idx >> (2 * b)) & 3);
    }
    for (uint32_t b = 0; b < k; b++) {
        uint32_t q = qs[b];
        if (m->bit_flip > 0.0 && zo_rng_f64(rng) < m->bit_flip) apply_pauli(s, q, 1);
        if (m->phase_flip > 0.0 && zo_rng_f64(rng) < m->phase_flip) apply_pauli(s, q, 3);
        if (m->amplitude_damping > 0.0) {
            double u = zo_rng_f64(rng);
            amplitude_damp(s, q, m->amplitude_damping, u);
        }
    }
}

static int readout_flip(const zo_noise *m, int bit, zo_rng *rng) {
    double p = bit ? m->readout_flip_1to0 : m->readout_flip_0to1;
    if (p > 0.0 && zo_rng_f64(rng) < p) return !bit;
    return bit;
}

static int noise_trivial(const zo_noise *m) {
    return !m || (m->depolarizing_1q == 0.0 && m->depolarizing_2q == 0.0 && m->bit_flip == 0.0 &&
                  m->phase_flip == 0.0 && m->amplitude_damping == 0.0 && m->readout_flip_0to1 == 0.0 &&
                  m->readout_flip_1to0 == 0.0);
}

/* ===================================================================== */
/* Executor (src/exec.rs:398-619).                                        */
/* ===================================================================== */

static void apply_op(zo_state *s, const zo_op *op) {
    if (op->kind == ZO_OP_UNITARY) zo_apply_unitary(s, op->qubits, op->k, op->data);
    else if (op->kind == ZO_OP_DIAG) zo_apply_diagonal(s, op->qubits, op->k, op->data);
    else if (op->kind == ZO_OP_CX) zo_apply_cx(s, op->control, op->target);
}

/* exec_shot_op (exec.rs:556-619) */
static void exec_shot_op(zo_state *s, const zo_op *op, const zo_noise *noise, zo_rng *rng, uint64_t *clbits) {
    if (op->has_if) {
        uint64_t mask = op->creg_len >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << op->creg_len) - 1);
        if (((*clbits >> op->creg_offset) & mask) != op->value) return;
    }
    switch (op->kind) {
    case ZO_OP_UNITARY:
    case ZO_OP_DIAG:
        apply_op(s, op);
        if (noise) apply_gate_noise(s, noise, op->qubits, op->k, rng);
        break;
    case ZO_OP_CX: {
        zo_apply_cx(s, op->control, op->target);
        if (noise) {
            uint32_t qs[2] = {op->control < op->target ? op->control : op->target,
                              op->control < op->target ? op->target : op->control};
            apply_gate_noise(s, noise, qs, 2, rng);
        }
        break;
    }
    case ZO_OP_MEASURE: {
        int bit = zo_measure(s, op->qubit, zo_rng_f64(rng));
        if (noise) bit = readout_flip(noise, bit, rng);
        *clbits = (*clbits & ~((uint64_t)1 << op->clbit)) | ((uint64_t)bit << op->clbit);
        break;
    }
    case ZO_OP_RESET: {
        if (zo_measure(s, op->qubit, zo_rng_f64(rng))) {
            zo_c64 x[4] = {cx(0, 0), cx(1.0, 0.0), cx(1.0, 0.0), cx(0, 0)};
            zo_apply_unitary(s, &op->qubit, 1, x);
        }
        break;
    }
    default:
        break;
    }
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

static long histogram(uint64_t *words, uint64_t n, uint64_t *keys, uint64_t *counts, size_t cap) {
    qsort(words, n, sizeof(uint64_t), cmp_u64);
    long m = 0;
    for (uint64_t i = 0; i < n;) {
        uint64_t j = i;
        while (j < n && words[j] == words[i]) j++;
        if ((size_t)m < cap) {
            keys[m] = words[i];
            counts[m] = j - i;
        }
        m++;
        i = j;
    }
    return m;
}

long zo_run(const zo_compiled *c, int prec, uint64_t shots, uint64_t seed, const zo_noise *noise, uint64_t *keys,
            uint64_t *counts, size_t cap, zo_c64 *sv_out) {
    if (noise_trivial(noise)) noise = NULL;
    if ((noise || c->dynamic) && sv_out) return -1;
    if (!noise && !c->dynamic) {
        /* run_sampled (exec.rs:407-452) */
        zo_state *s = zo_state_new(c->n_qubits, prec);
        if (!s) return -1;
        for (size_t i = 0; i < c->nops; i++) apply_op(s, &c->ops[i]);
        if (sv_out) zo_statevector(s, sv_out);
        long m = 0;
        if (c->nfinal > 0 && shots > 0) {
            uint64_t *smp = (uint64_t *)malloc(shots * sizeof(uint64_t));
            zo_sample(s, shots, zo_splitmix64(seed), smp);
            for (uint64_t i = 0; i < shots; i++) {
                uint64_t basis = smp[i], cl = 0;
                for (size_t f = 0; f < c->nfinal; f++) {
                    uint64_t bit = (basis >> c->fq[f]) & 1;
                    cl = (cl & ~((uint64_t)1 << c->fc[f])) | (bit << c->fc[f]);
                }
                smp[i] = cl;
            }
            m = histogram(smp, shots, keys, counts, cap);
            free(smp);
        }
        zo_state_free(s);
        return m;
    }
    /* run_per_shot (exec.rs:459-549) */
    if (!c->dynamic && c->nfinal == 0) return 0;
    uint64_t *words = (uint64_t *)malloc((shots ? shots : 1) * sizeof(uint64_t));
    size_t amps = (size_t)1 << c->n_qubits;
    int parallel = shots > 1 && amps <= ((size_t)1 << 22);
#pragma omp parallel if (parallel)
    {
        zo_state *s = zo_state_new(c->n_qubits, prec);
#pragma omp for schedule(dynamic, 8)
        for (uint64_t shot = 0; shot < shots; shot++) {
            zo_reset_all(s);
            zo_rng rng;
            zo_rng_seed(&rng, zo_splitmix64(seed ^ shot));
            uint64_t cl = 0;
            for (size_t i = 0; i < c->nops; i++) exec_shot_op(s, &c->ops[i], noise, &rng, &cl);
            for (size_t f = 0; f < c->nfinal; f++) {
                int bit = zo_measure(s, c->fq[f], zo_rng_f64(&rng));
                if (noise) bit = readout_flip(noise, bit, &rng);
                cl = (cl & ~((uint64_t)1 << c->fc[f])) | ((uint64_t)bit << c->fc[f]);
            }
            words[shot] = cl;
        }
        zo_state_free(s);
    }
    long m = histogram(words, shots, keys, counts, cap);
    free(words);
    return m;
}

/* ===================================================================== */
/* mem.rs (state_bytes :79-81, max_qubits :84-94)                         */
/* ===================================================================== */

uint64_t zo_state_bytes(uint32_t n, int prec) { return ((uint64_t)1 << n) * (prec == 32 ? 8u : 16u); }

uint32_t zo_max_qubits(uint64_t budget, int prec) {
    uint32_t n = 0;
    while ((((unsigned __int128)1) << (n + 1)) * (unsigned __int128)(prec == 32 ? 8 : 16) <= budget) {
        n++;
        if (n >= 60) break;
    }
    return n;
}

/* ===================================================================== */
/* Independent dense simulator (tests/reference.rs:69-116).               */
/* ===================================================================== */

void zo_refsim_apply(zo_c64 *amps, uint32_t n, const uint32_t *qs, uint32_t k, const zo_c64 *mat) {
    size_t dim = (size_t)1 << k, mask = 0, offset[128];
    for (uint32_t b = 0; b < k; b++) mask |= (size_t)1 << qs[b];
    for (size_t m = 0; m < dim; m++) {
        size_t o = 0;
        for (uint32_t b = 0; b < k; b++)
            if ((m >> b) & 1) o += (size_t)1 << qs[b];
        offset[m] = o;
    }
    zo_c64 old[128];
    for (size_t base = 0; base < ((size_t)1 << n); base++) {
        if (base & mask) continue;
        for (size_t m = 0; m < dim; m++) old[m] = amps[base + offset[m]];
        for (size_t l = 0; l < dim; l++) {
            zo_c64 acc = cx(0.0, 0.0);
            for (size_t m = 0; m < dim; m++) acc = cadd(acc, cmul(mat[l * dim + m], old[m]));
            amps[base + offset[l]] = acc;
        }
    }
}
