// C ABI of the backend (include/zeno_cuda.h): state lifecycle, argument
// validation, op dispatch onto the gate kernels, reductions, the sampler's
// host half, and HBM capacity planning.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "zc_internal.h"
#include "zc_rng.h"
#include "zc_sweep.h"

namespace zc {

static thread_local std::string g_err;

const char *const kKernelNames[K_NKINDS] = {"1q",         "kq",         "diag1",       "diagk",    "cx",
                                            "swap",       "sweep",      "chunk_sums",  "serial_sum", "sample_scan",
                                            "collapse",   "reset",      "trajectories", "tc_block"};

ProfScope::ProfScope(zc_state *s, int kind, double bytes) : st(s) {
    if (!st || !st->prof) return;
    cudaEvent_t ev[2];
    for (int i = 0; i < 2; i++) {
        if (!st->prof_pool.empty()) {
            ev[i] = st->prof_pool.back();
            st->prof_pool.pop_back();
        } else if (cudaEventCreate(&ev[i]) != cudaSuccess) {
            return;
        }
    }
    cudaEventRecord(ev[0], st->stream);
    st->prof_recs.push_back(ProfRec{kind, bytes, ev[0], ev[1]});
    idx = (long)st->prof_recs.size() - 1;
}

ProfScope::~ProfScope() {
    if (idx >= 0) cudaEventRecord(st->prof_recs[idx].b, st->stream);
}

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *where) {
    g_err = std::string("CUDA error in ") + where + ": " + cudaGetErrorString(e);
    return ZC_ERR_CUDA;
}

static std::string human_bytes(double b) {
    const char *units[] = {"B", "KiB", "MiB", "GiB", "TiB"};
    int u = 0;
    while (b >= 1024.0 && u < 4) {
        b /= 1024.0;
        u++;
    }
    char buf[64];
    if (u == 0)
        snprintf(buf, sizeof buf, "%.0f B", b);
    else
        snprintf(buf, sizeof buf, "%.1f %s", b, units[u]);
    return buf;
}

static constexpr size_t kArenaBytes = 32u << 20;

// Copy `bytes` into the device parameter ring and return its device address.
int arena_put(zc_state *st, const void *src, size_t bytes, const void **dev) {
    Arena &a = st->arena;
    const size_t need = (bytes + 255) & ~(size_t)255;
    if (need > a.cap) return fail(ZC_ERR_INVALID, "op table larger than the parameter arena");
    if (a.head + need > a.cap) {
        ZC_CUDA(cudaStreamSynchronize(st->stream));
        a.head = 0;
    }
    memcpy(a.host + a.head, src, bytes);
    ZC_CUDA(cudaMemcpyAsync(a.dev + a.head, a.host + a.head, bytes, cudaMemcpyHostToDevice, st->stream));
    *dev = a.dev + a.head;
    a.head += need;
    return ZC_OK;
}

// Stage a complex table (interleaved c64) as split T arrays [re..., im...].
static int stage_table(zc_state *st, const double *c64, size_t count, const void **dev) {
    if (st->prec == 64) {
        std::vector<double> t(2 * count);
        for (size_t i = 0; i < count; i++) {
            t[i] = c64[2 * i];
            t[count + i] = c64[2 * i + 1];
        }
        return arena_put(st, t.data(), t.size() * sizeof(double), dev);
    }
    std::vector<float> t(2 * count);
    for (size_t i = 0; i < count; i++) {
        t[i] = (float)c64[2 * i];
        t[count + i] = (float)c64[2 * i + 1];
    }
    return arena_put(st, t.data(), t.size() * sizeof(float), dev);
}

static int check_support(const zc_state *st, const uint32_t *qs, uint32_t k, uint32_t kmax, const char *what) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    if (k < 1 || k > kmax) return fail(ZC_ERR_INVALID, std::string(what) + ": support size out of range");
    if (!qs) return fail(ZC_ERR_INVALID, std::string(what) + ": null qubit list");
    for (uint32_t i = 0; i < k; i++) {
        if (qs[i] >= st->n) return fail(ZC_ERR_INVALID, std::string(what) + ": qubit out of range");
        if (i && qs[i] <= qs[i - 1])
            return fail(ZC_ERR_INVALID, std::string(what) + ": qubits must be sorted and distinct");
    }
    return ZC_OK;
}

static inline bool exact(const zc_state *st) { return (st->flags & ZC_FLAG_FAST) == 0; }


static int sync_read_scalar(zc_state *st, double *out) {
    ZC_CUDA(cudaMemcpyAsync(st->h_scalar, st->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    *out = *st->h_scalar;
    return check_device_error(st);  // a kernel that gave up leaves a wrong state behind
}

static int grow(void **p, size_t *cap, size_t need) {
    if (need <= *cap) return ZC_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    ZC_CUDA(cudaMalloc(p, need));
    *cap = need;
    return ZC_OK;
}


// ------------------------------------------------------------------ scheduling

static constexpr size_t kQueueWindow = 2048;  // ops examined per sweep plan
static constexpr size_t kQueueFlushAt = 8192; // queue length that forces a flush
static constexpr uint32_t kMinSweepQubits = 14;

int launch_single(zc_state *st, const QOp &op) {
    const bool ex = exact(st);
    switch (op.kind) {
        case Q_UNITARY: {
            if (op.k == 1) return launch_1q(st, op.qs[0], op.data.data(), ex);
            if (op.k >= 3 && st->prec == 32 && (st->flags & ZC_FLAG_TENSOR))
                return launch_block_tc(st, op.qs, op.k, op.data.data());
            const void *dev = nullptr;
            if (st->prec == 64 && !ex) {  // fast f64: double-float on the FP32 pipe
                const size_t cnt = (size_t)1 << (2 * op.k);
                std::vector<float> t(4 * cnt);
                for (size_t i = 0; i < cnt; i++) {
                    for (int part = 0; part < 2; part++) {  // re, im: hi = nearest float, lo = the rest
                        const double x = op.data[2 * i + part];
                        const float hi = (float)x;
                        t[4 * i + 2 * part] = hi;
                        t[4 * i + 2 * part + 1] = (float)(x - (double)hi);
                    }
                }
                int rc = arena_put(st, t.data(), t.size() * sizeof(float), &dev);
                if (rc) return rc;
                return launch_kq_df(st, op.qs, op.k, dev);
            }
            int rc = stage_table(st, op.data.data(), (size_t)1 << (2 * op.k), &dev);
            if (rc) return rc;
            return launch_kq(st, op.qs, op.k, dev, ex);
        }
        case Q_DIAG: {
            if (op.k == 1) return launch_diag1(st, op.qs[0], op.data.data(), ex);
            const void *dev = nullptr;
            int rc = stage_table(st, op.data.data(), (size_t)1 << op.k, &dev);
            if (rc) return rc;
            return launch_diagk(st, op.qs, op.k, dev, ex);
        }
        case Q_CX:
            return launch_cx(st, op.a, op.b);
        default:
            return launch_swap(st, op.a, op.b);
    }
}

static uint64_t touch_mask(const QOp &op) {
    if (op.kind == Q_CX || op.kind == Q_SWAP) return (1ull << op.a) | (1ull << op.b);
    uint64_t m = 0;
    for (uint32_t i = 0; i < op.k; i++) m |= 1ull << op.qs[i];
    return m;
}

// Qubits that must be local for `op` to run inside a sweep.
static uint64_t need_mask(const QOp &op) {
    switch (op.kind) {
        case Q_UNITARY: return 1ull << op.qs[0];
        case Q_DIAG: return 0;
        case Q_CX: return 1ull << op.b;
        default: return (1ull << op.a) | (1ull << op.b);
    }
}

static bool sweepable(const QOp &op) { return !(op.kind == Q_UNITARY && op.k > 1); }

struct SweepShape {
    uint32_t L, Hcap;
};

static SweepShape shape_for(const zc_state *st) {
    const uint32_t L = std::min<uint32_t>(st->n, st->prec == 64 ? 5 : 6);  // 256-byte rows
    const uint32_t Tmax = st->prec == 64 ? 12 : 13;                       // 64 KiB per tile buffer
    uint32_t Hcap = std::min<uint32_t>(Tmax - L, st->n - L);
    if (st->sweep_high) return SweepShape{L, std::min<uint32_t>(Hcap, st->sweep_high)};  // tuned
    // keep at least ~2 tiles per SM so every SM streams
    uint32_t tiles_log2 = 0;
    while ((1u << tiles_log2) < (uint32_t)(2 * st->num_sms)) tiles_log2++;
    if (st->n - L > tiles_log2) Hcap = std::min<uint32_t>(Hcap, st->n - L - tiles_log2);
    else Hcap = 0;
    return SweepShape{L, Hcap};
}

static uint32_t loc_of(uint32_t q, uint32_t L, const std::vector<uint32_t> &highs) {
    if (q < L) return q;
    for (size_t j = 0; j < highs.size(); j++)
        if (highs[j] == q) return L + (uint32_t)j;
    return kOuterFlag | q;
}

// Choose the ops of one sweep from the queue front (see the scheduling
// rules above). Fills `plan` and returns how many ops it took; 0 or 1 means
// the front op should simply run on its own.
size_t plan_sweep(uint32_t n, int prec, bool ex, uint32_t L, uint32_t Hcap, const std::vector<QOp> &q,
                  SweepPlan *plan) {
    const uint64_t low_mask = L >= 64 ? ~0ull : ((1ull << L) - 1);
    uint64_t blocked = 0, highs_mask = 0;
    uint32_t nhigh = 0;
    bool arith_deferred = false;
    std::vector<size_t> &taken = plan->taken;
    taken.clear();
    const size_t window = std::min(q.size(), kQueueWindow);
    // Under double-float lowering a diagonal joins the pending tables and
    // becomes a micro-op only when flushed, so it does not count against the
    // micro-op budget here (the lowered count is checked below).
    const bool df_lowering = !ex && prec == 64;
    size_t counted = 0;
    for (size_t i = 0; i < window && counted < (size_t)kMaxMicroOps && taken.size() < 4 * (size_t)kMaxMicroOps;
         i++) {
        const QOp &op = q[i];
        const uint64_t touch = touch_mask(op);
        const bool arith = op.kind == Q_UNITARY || op.kind == Q_DIAG;
        bool defer = (touch & blocked) != 0 || (ex && arith && arith_deferred) || !sweepable(op);
        uint64_t need = 0;
        if (!defer) {
            need = need_mask(op) & ~low_mask & ~highs_mask;
            if (nhigh + (uint32_t)__builtin_popcountll(need) > Hcap) defer = true;
        }
        if (defer) {
            blocked |= touch;
            arith_deferred |= arith;
            continue;
        }
        highs_mask |= need;
        nhigh += (uint32_t)__builtin_popcountll(need);
        taken.push_back(i);
        counted += !(df_lowering && op.kind == Q_DIAG);
    }
    if (taken.size() <= 1) return taken.size();
    // pad the tile with further high qubits up to the cap (no effect on results)
    for (uint32_t b = L; b < n && nhigh < Hcap; b++)
        if (!((highs_mask >> b) & 1)) {
            highs_mask |= 1ull << b;
            nhigh++;
        }
    std::vector<uint32_t> highs;
    for (uint32_t b = 0; b < n; b++)
        if ((highs_mask >> b) & 1) highs.push_back(b);
    SweepGeom &g = plan->g;
    g = SweepGeom{};
    g.n = n;
    g.L = L;
    g.H = (uint32_t)highs.size();
    for (size_t j = 0; j < highs.size(); j++) g.hpos[j] = highs[j];
    g.ntiles = 1ull << (n - g.L - g.H);
    // Order of the micro-ops. Exact mode keeps program order (reordering two
    // gates changes the rounding). Fast mode lets ops on disjoint qubits
    // commute: one-qubit ops on distinct qubits are emitted back to back, in
    // runs the size of the kernel's register groups (three for the rotations
    // of lowered f64 sweeps, else two: f32 groups of two move element pairs
    // as 8-byte vectors), so the kernel applies each run in one register pass.
    const size_t run_cap = prec == 32 ? 2 : (prec == 64 && !df_lowering ? 2 : 3);
    const bool df = df_lowering;
    std::vector<LoweredOp> low;
    for (;;) {
    std::vector<size_t> order(taken.size());
    for (size_t t = 0; t < taken.size(); t++) order[t] = t;
    if (!ex) {
        const size_t m = taken.size();
        std::vector<char> done(m, 0);
        auto ready = [&](size_t i) {
            for (size_t j = 0; j < i; j++)
                if (!done[j] && (touch_mask(q[taken[j]]) & touch_mask(q[taken[i]]))) return false;
            return true;
        };
        auto is1q = [&](size_t i) { return q[taken[i]].kind == Q_UNITARY && q[taken[i]].k == 1; };
        order.clear();
        uint64_t cx_targets = 0;  // targets of the CX ops since the last run
        while (order.size() < m) {
            // ready one-qubit ops on distinct qubits, program order; those on
            // targets of the CX ops just emitted first (the kernel folds a CX
            // into the register group that holds its target)
            std::vector<size_t> run;
            uint64_t used = 0;
            for (int pass = 0; pass < 2; pass++)
                for (size_t i = 0; i < m && run.size() < run_cap; i++) {
                    if (done[i] || !is1q(i) || !ready(i)) continue;
                    const uint32_t qb = q[taken[i]].qs[0];
                    if ((used >> qb) & 1) continue;
                    if (pass == 0 && !((cx_targets >> qb) & 1)) continue;
                    run.push_back(i);
                    used |= 1ull << qb;
                }
            std::sort(run.begin(), run.end());
            // a full run goes out at once; otherwise a ready op of another
            // kind goes first (it can make more one-qubit ops ready), and a
            // short run only when nothing else is ready
            bool emitted = false;
            if (run.size() < run_cap)
                for (size_t i = 0; i < m && !emitted; i++)
                    if (!done[i] && !is1q(i) && ready(i)) {
                        done[i] = 1;
                        order.push_back(i);
                        emitted = true;
                        if (q[taken[i]].kind == Q_CX) cx_targets |= 1ull << q[taken[i]].b;
                    }
            if (emitted) continue;
            for (size_t i : run) {
                done[i] = 1;
                order.push_back(i);
            }
            cx_targets = 0;
        }
    }
    // Lowering: double-float sweeps of f64 states rewrite one-qubit gates as
    // diagonal * real * diagonal and merge the diagonals; other policies
    // encode the ops as they are.
    low.clear();
    plan->carry.clear();
    if (df) {
        std::vector<const QOp *> seq;
        for (size_t t : order) seq.push_back(&q[taken[t]]);
        lower_df(seq, 2, &low, &plan->carry);
    } else {
        for (size_t t : order) {
            const QOp &op = q[taken[t]];
            LoweredOp o{};
            if (op.kind == Q_UNITARY) {
                o.kind = MOP_U1;
                o.a = op.qs[0];
                for (int i = 0; i < 8; i++) o.m[i] = op.data[i];
            } else if (op.kind == Q_DIAG) {
                o.kind = MOP_DK;
                o.sup.assign(op.qs, op.qs + op.k);
                o.tab = op.data;
            } else {
                o.kind = op.kind == Q_CX ? MOP_CX : MOP_SWAP;
                o.a = op.a;
                o.b = op.b;
            }
            low.push_back(std::move(o));
        }
    }
    if (low.size() <= (size_t)kMaxMicroOps) break;
    // lowering added table ops: take fewer queue ops (dropping the last
    // taken op never breaks an ordering constraint)
    taken.pop_back();
    if (taken.size() <= 1) {
        plan->carry.clear();
        return taken.size();
    }
    }
    std::vector<MicroOp> &mops = plan->mops;
    std::vector<char> &tables = plan->tables;
    mops.assign(low.size(), MicroOp{});
    tables.clear();
    const size_t es = prec / 8;
    for (size_t t = 0; t < low.size(); t++) {
        const LoweredOp &op = low[t];
        MicroOp &m = mops[t];
        if (op.kind == MOP_U1 || op.kind == MOP_R1 || op.kind == MOP_RT) {
            m.kind = op.kind;
            m.a = loc_of(op.a, g.L, highs);
            if (op.kind == MOP_RT) m.b = op.b;  // form
            for (int i = 0; i < 8; i++) m.m[i] = op.m[i];
        } else if (op.kind == MOP_DK && op.sup.size() == 1 && !df) {  // double-float: tables ride in groups
            m.kind = MOP_D1;
            m.a = loc_of(op.sup[0], g.L, highs);
            for (int i = 0; i < 4; i++) m.m[i] = op.tab[i];
        } else if (op.kind == MOP_DK) {
            m.kind = MOP_DK;
            m.k = (uint32_t)op.sup.size();
            for (uint32_t b = 0; b < m.k; b++) m.loc[b] = loc_of(op.sup[b], g.L, highs);
            const size_t dim = (size_t)1 << m.k;
            size_t off = (tables.size() + 15) & ~(size_t)15;
            tables.resize(off + 2 * dim * es);
            for (size_t j = 0; j < dim; j++) {
                const double xr = op.tab[2 * j], xi = op.tab[2 * j + 1];
                if (df) {  // (re hi, re lo, im hi, im lo)
                    float *e = (float *)(tables.data() + off) + 4 * j;
                    e[0] = (float)xr;
                    e[1] = (float)(xr - (double)e[0]);
                    e[2] = (float)xi;
                    e[3] = (float)(xi - (double)e[2]);
                } else if (es == 8) {  // (re, im) pairs: one 16-byte load per entry
                    ((double *)(tables.data() + off))[2 * j] = xr;
                    ((double *)(tables.data() + off))[2 * j + 1] = xi;
                } else {
                    ((float *)(tables.data() + off))[2 * j] = (float)xr;
                    ((float *)(tables.data() + off))[2 * j + 1] = (float)xi;
                }
            }
            m.table = off;
        } else {
            m.kind = op.kind;
            m.a = loc_of(op.a, g.L, highs);
            m.b = loc_of(op.b, g.L, highs);
        }
    }
    return taken.size();
}

// Remove the ops at the (ascending) indices `taken`, keeping the rest in order.
void erase_taken(std::vector<QOp> &q, const std::vector<size_t> &taken) {
    std::vector<QOp> rest;
    rest.reserve(q.size() - taken.size());
    size_t ti = 0;
    for (size_t i = 0; i < q.size(); i++) {
        if (ti < taken.size() && taken[ti] == i) {
            ti++;
            continue;
        }
        rest.push_back(std::move(q[i]));
    }
    q.swap(rest);
}

// The carried diagonals act after every op the sweep took and touch only
// qubits those ops touched; no op deferred ahead of them touches those qubits,
// so the queue front is their place in program order.
void consume_plan(std::vector<QOp> &q, SweepPlan &plan) {
    erase_taken(q, plan.taken);
    if (!plan.carry.empty()) {
        q.insert(q.begin(), std::make_move_iterator(plan.carry.begin()), std::make_move_iterator(plan.carry.end()));
        plan.carry.clear();
    }
}

static bool sweepable(const QOp &op);
static bool sweeps_enabled(const zc_state *st);

// Before any kernel other than a sweep: a state that double-float sweeps
// left as packed float pairs goes back to f64.
static int settle_form(zc_state *st) {
    if (!st->df_resident) return ZC_OK;
    st->df_resident = false;
    return launch_df_to_f64(st);
}

// Plan and launch one sweep starting at the queue front; erases what ran.
static int run_one_sweep(zc_state *st) {
    std::vector<QOp> &q = st->queue;
    const SweepShape sh = shape_for(st);
    SweepPlan plan;
    if (plan_sweep(st->n, st->prec, exact(st), sh.L, sh.Hcap, q, &plan) <= 1) {
        // nothing to batch: the per-op kernel is the same work
        int rc = settle_form(st);
        if (rc) return rc;
        rc = launch_single(st, q.front());
        q.erase(q.begin());
        return rc;
    }
    const size_t ops_bytes = plan.mops.size() * sizeof(MicroOp);
    const size_t tab_off = (ops_bytes + 255) & ~(size_t)255;
    std::vector<char> blob(tab_off + plan.tables.size());
    memcpy(blob.data(), plan.mops.data(), ops_bytes);
    if (!plan.tables.empty()) memcpy(blob.data() + tab_off, plan.tables.data(), plan.tables.size());
    const void *dev = nullptr;
    int rc = arena_put(st, blob.data(), blob.size(), &dev);
    if (rc) return rc;
    consume_plan(q, plan);
    // Fast f64: consecutive sweeps of one flush hand the state over as
    // (hi, lo) float pairs; the last one (nothing sweepable queued behind
    // it) rounds it back to f64.
    const bool df = st->prec == 64 && !exact(st);
    const bool out_df = df && !q.empty() && sweepable(q.front());
    plan.g.form = (st->df_resident ? kFormInDf : 0u) | (out_df ? kFormOutDf : 0u);
    rc = launch_sweep(st, plan.g, (const MicroOp *)dev, (int)plan.mops.size(), (const char *)dev + tab_off,
                      exact(st));
    st->df_resident = out_df;
    for (const MicroOp &m : plan.mops) st->ctr.micro_ops[m.kind & 7]++;
    return rc;
}

static bool sweeps_enabled(const zc_state *st) {
    if (st->flags & ZC_FLAG_NO_SWEEPS) return false;
    if (st->flags & ZC_FLAG_FORCE_SWEEPS) return st->n >= 3;
    return st->n >= kMinSweepQubits;
}

// Launch everything queued (program order preserved where results depend on it).
static int flush(zc_state *st) {
    int rc = ZC_OK;
    while (!st->queue.empty() && rc == ZC_OK) {
        if (!sweeps_enabled(st) || !sweepable(st->queue.front())) {
            rc = settle_form(st);
            if (rc == ZC_OK) rc = launch_single(st, st->queue.front());
            st->queue.erase(st->queue.begin());
            continue;
        }
        rc = run_one_sweep(st);
    }
    st->queue.clear();
    const int rc2 = settle_form(st);  // every other entry point sees f64
    return rc ? rc : rc2;
}

static int enqueue(zc_state *st, QOp &&op) {
    st->ctr.ops++;
    if (!sweeps_enabled(st)) return launch_single(st, op);
    st->queue.push_back(std::move(op));
    if (st->queue.size() >= kQueueFlushAt) return flush(st);
    return ZC_OK;
}

int check_device_error(zc_state *st) {
    int h[kErrWords] = {};
    ZC_CUDA(cudaMemcpyAsync(h, st->d_err, sizeof(h), cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    if (h[0]) {
        cudaMemsetAsync(st->d_err, 0, sizeof(h), st->stream);
        if (h[0] == 3)
            return fail(ZC_ERR_CUDA, "tensor-core block kernel gave up waiting for a copy or an MMA (device wait limit)");
        char buf[320];
        snprintf(buf, sizeof(buf),
                 "sweep kernel %s (cta %d tile %d phase %d barrier %08x%08x L %d H %d ops %d tiles done %d index %08x)",
                 h[0] == 1 ? "gave up waiting for a bulk copy (device wait limit reached)"
                           : "found a tile index out of range",
                 h[1], h[2], h[3], (unsigned)h[5], (unsigned)h[4], h[6], h[7], h[8], h[9], (unsigned)h[10]);
        return fail(ZC_ERR_CUDA, buf);
    }
    return ZC_OK;
}

// Sampler host half (src/sample.rs:51-62), exactly as the reference orders
// it: serial prefix of the chunk masses, `shots` serial draws scaled by the
// total, ascending sort, and the routing of draws to chunks
// (partition_point(u < cum_before[c])).
void sample_route(const double *sums, size_t nch, uint64_t len, uint64_t shots, uint64_t seed, SampleRoute *r) {
    std::vector<double> cum(nch + 1);
    cum[0] = 0.0;
    for (size_t c = 0; c < nch; c++) cum[c + 1] = cum[c] + sums[c];
    const double total = cum[nch];
    Xoshiro rng(seed);
    r->us.resize(shots);
    for (uint64_t i = 0; i < shots; i++) r->us[i] = rng.f64() * total;
    std::sort(r->us.begin(), r->us.end());
    r->touched.clear();
    size_t prev = std::lower_bound(r->us.begin(), r->us.end(), cum[0]) - r->us.begin();
    for (size_t c = 0; c < nch; c++) {
        const size_t next = std::lower_bound(r->us.begin(), r->us.end(), cum[c + 1]) - r->us.begin();
        if (prev < next) r->touched.push_back(SampleChunk{c, prev, next, cum[c]});
        prev = next;
    }
    r->chunk_len = len < (1ull << kSampleChunkLog2) ? len : (1ull << kSampleChunkLog2);
}

static size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t sample_pass2_bytes(const zc_state *st, const SampleRoute &r) {
    return up256(r.us.size() * sizeof(uint64_t)) + up256(r.us.size() * sizeof(double)) +
           up256(r.touched.size() * sizeof(SampleChunk)) + sample_scan_scratch(r.touched.size(), r.chunk_len, exact(st));
}

// Pass 2, asynchronous. d_work (sample_pass2_bytes(st, r) bytes, 256-aligned)
// holds [indices | draws | touched chunks | rescan scratch]; draws and chunk
// lists small enough travel through the pinned parameter ring, larger ones
// are copied from pageable memory (which waits for the stream).
int sample_launch_pass2(zc_state *st, const SampleRoute &r, char *d_work, uint64_t **d_out) {
    const size_t shots = r.us.size();
    uint64_t *out = (uint64_t *)d_work;
    *d_out = out;
    if (shots == 0) return ZC_OK;
    const size_t out_b = up256(shots * sizeof(uint64_t)), us_b = up256(shots * sizeof(double));
    const size_t cs_b = up256(r.touched.size() * sizeof(SampleChunk));
    const size_t cs_n = r.touched.size() * sizeof(SampleChunk);
    const void *d_us = d_work + out_b, *d_cs = d_work + out_b + us_b;
    int rc = ZC_OK;
    // Through the ring only when both fit in a quarter of it: if the second
    // put wraps, the first began past three quarters, beyond the reach of the
    // second (placed at offset 0), so the kernel reads both intact.
    if (shots * sizeof(double) + cs_n <= st->arena.cap / 4) {
        rc = arena_put(st, r.us.data(), shots * sizeof(double), &d_us);
        if (rc == ZC_OK && cs_n) rc = arena_put(st, r.touched.data(), cs_n, &d_cs);
        if (rc) return rc;
    } else {
        ZC_CUDA(cudaMemcpyAsync((void *)d_us, r.us.data(), shots * sizeof(double), cudaMemcpyHostToDevice, st->stream));
        if (cs_n)
            ZC_CUDA(cudaMemcpyAsync((void *)d_cs, r.touched.data(), cs_n, cudaMemcpyHostToDevice, st->stream));
    }
    ZC_CUDA(cudaMemsetAsync(out, 0, shots * sizeof(uint64_t), st->stream));
    char *scratch = d_work + out_b + us_b + cs_b;
    return launch_sample_scan(st, (const SampleChunk *)d_cs, r.touched.size(), (const double *)d_us, out, r.chunk_len,
                              exact(st), scratch);
}

}  // namespace zc

using namespace zc;

extern "C" {

const char *zc_last_error(void) { return g_err.c_str(); }

uint64_t zc_state_bytes(uint32_t n, int prec) { return (n >= 64 ? 0 : (1ull << n)) * (prec == 32 ? 8u : 16u); }

uint32_t zc_max_qubits(uint64_t budget, int prec) {
    uint32_t n = 0;
    while ((((unsigned __int128)1) << (n + 1)) * (unsigned __int128)(prec == 32 ? 8 : 16) <= budget) {
        n++;
        if (n >= 60) break;
    }
    return n;
}

// physical_ram_bytes (src/mem.rs:9-16) for the device: ZENO_MEM_BYTES
// pretends to be a device of that many bytes, else the device's total HBM.
static int device_memory(uint64_t *bytes) {
    const char *env = getenv("ZENO_MEM_BYTES");
    if (env && *env) {
        char *end = nullptr;
        unsigned long long v = strtoull(env, &end, 10);
        if (end && *end == 0) {
            *bytes = v;
            return ZC_OK;
        }
    }
    size_t free_b = 0, total_b = 0;
    cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemGetInfo");
    *bytes = total_b;
    return ZC_OK;
}

// budget_bytes without an explicit limit (src/mem.rs:104-111).
int zc_device_budget(double fraction, uint64_t *bytes) {
    if (!bytes) return fail(ZC_ERR_INVALID, "null output");
    uint64_t mem = 0;
    const int rc = device_memory(&mem);
    if (rc) return rc;
    *bytes = (uint64_t)((double)mem * fraction);
    return ZC_OK;
}

int zc_device_memory(uint64_t *bytes) {
    if (!bytes) return fail(ZC_ERR_INVALID, "null output");
    return device_memory(bytes);
}

int zc_device_info(zc_device *out) {
    if (!out) return fail(ZC_ERR_INVALID, "null output");
    memset(out, 0, sizeof *out);
    int dev = 0;
    ZC_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    ZC_CUDA(cudaGetDeviceProperties(&prop, dev));
    snprintf(out->name, sizeof out->name, "%s", prop.name);
    out->sms = (uint32_t)prop.multiProcessorCount;
    out->cc_major = (uint32_t)prop.major;
    out->cc_minor = (uint32_t)prop.minor;
    size_t free_b = 0, total_b = 0;
    ZC_CUDA(cudaMemGetInfo(&free_b, &total_b));
    out->hbm_bytes = total_b;
    out->free_bytes = free_b;
    out->l2_bytes = (uint64_t)prop.l2CacheSize;
    return ZC_OK;
}

int zc_create(uint32_t n, int prec, zc_state **out) { return zc_create_ex(n, prec, ZC_FLAG_EXACT, out); }

}  // extern "C"

namespace zc {

// mem::plan (src/mem.rs:114-131): refuse a state above the budget, with the
// text of zeno's Error::Memory.
int plan_state(uint32_t n, int prec, uint64_t budget) {
    const uint64_t need = zc_state_bytes(n, prec);
    if (need > budget) {
        char buf[256];
        snprintf(buf, sizeof buf,
                 "state vector for %u qubits at f%d needs %s but the budget is %s (max %u qubits at this "
                 "precision; raise --mem-limit or lower qubits)",
                 n, prec, human_bytes((double)need).c_str(), human_bytes((double)budget).c_str(),
                 zc_max_qubits(budget, prec));
        return fail(ZC_ERR_MEMORY, buf);
    }
    return ZC_OK;
}

}  // namespace zc

extern "C" int zc_create_ex(uint32_t n, int prec, uint32_t flags, zc_state **out) {
    if (!out) return fail(ZC_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (prec != 32 && prec != 64) return fail(ZC_ERR_INVALID, "precision_bits must be 32 or 64");
    if (n < 1 || n > 48) return fail(ZC_ERR_INVALID, "qubit count must be in 1..=48");
    uint64_t budget = 0;
    int rc = zc_device_budget(0.75, &budget);
    if (rc) return rc;
    return create_state(n, prec, flags, budget, out);
}

namespace zc {
namespace {

// A state's buffers that do not depend on its size: stream, parameter ring
// (pinned host + device), scalar and error words, sampler scratch. Released
// states hand them to a small per-process cache (at most kKitCache, per
// device) and new states take them from it, so a run of short-lived states —
// one zc_run per circuit — does not pay a 32 MiB pinned allocation, a device
// allocation and their frees every time. The cache holds up to
// kKitCache x 64 MiB (half pinned host, half device) until the process exits.
struct Kit {
    int device = 0;
    cudaStream_t stream = nullptr;
    Arena arena;
    double *d_scalar = nullptr, *h_scalar = nullptr;
    int *d_err = nullptr;
    double *d_part = nullptr;
    size_t part_cap = 0;
    void *d_samp = nullptr;
    size_t samp_cap = 0;
};
constexpr size_t kKitCache = 4;
std::mutex g_kit_mu;
std::vector<Kit> g_kits;

void free_kit(Kit &k) {
    if (k.stream) cudaStreamSynchronize(k.stream);
    if (k.arena.host) cudaFreeHost(k.arena.host);
    if (k.arena.dev) cudaFree(k.arena.dev);
    if (k.d_part) cudaFree(k.d_part);
    if (k.d_scalar) cudaFree(k.d_scalar);
    if (k.h_scalar) cudaFreeHost(k.h_scalar);
    if (k.d_samp) cudaFree(k.d_samp);
    if (k.d_err) cudaFree(k.d_err);
    if (k.stream) cudaStreamDestroy(k.stream);
    k = Kit{};
}

bool take_kit(int device, Kit *out) {
    std::lock_guard<std::mutex> lk(g_kit_mu);
    for (size_t i = 0; i < g_kits.size(); i++)
        if (g_kits[i].device == device) {
            *out = g_kits[i];
            g_kits.erase(g_kits.begin() + (long)i);
            return true;
        }
    return false;
}

// Returns false when the cache is full (the caller frees the kit).
bool give_kit(const Kit &k) {
    std::lock_guard<std::mutex> lk(g_kit_mu);
    if (g_kits.size() >= kKitCache) return false;
    g_kits.push_back(k);
    return true;
}

}  // namespace
}  // namespace zc

int zc::create_state(uint32_t n, int prec, uint32_t flags, uint64_t budget, zc_state **out) {
    if (!out) return fail(ZC_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (prec != 32 && prec != 64) return fail(ZC_ERR_INVALID, "precision_bits must be 32 or 64");
    if (n < 1 || n > 48) return fail(ZC_ERR_INVALID, "qubit count must be in 1..=48");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(ZC_ERR_UNSUPPORTED, std::string("no usable CUDA device: ") + cudaGetErrorString(e));
    int rc = plan_state(n, prec, budget);
    if (rc) return rc;
    zc_state *st = new zc_state();
    st->n = n;
    st->prec = prec;
    st->flags = flags;
    st->device = dev;
    st->len = 1ull << n;
    st->name = prec == 64 ? "cuda-f64" : "cuda-f32";
    cudaDeviceGetAttribute(&st->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (st->num_sms <= 0) st->num_sms = 1;
    const size_t bytes = st->len * (prec / 8);
#define TRY(call)                          \
    do {                                   \
        cudaError_t e_ = (call);           \
        if (e_ != cudaSuccess) {           \
            int r_ = cuda_fail(e_, #call); \
            zc_destroy(st);                \
            return r_;                     \
        }                                  \
    } while (0)
    Kit kit;
    if (take_kit(dev, &kit)) {  // stream, ring, scalars, sampler scratch of a released state
        st->stream = kit.stream;
        st->arena = kit.arena;
        st->arena.head = 0;
        st->d_scalar = kit.d_scalar;
        st->h_scalar = kit.h_scalar;
        st->d_err = kit.d_err;
        st->d_part = kit.d_part;
        st->part_cap = kit.part_cap;
        st->d_samp = kit.d_samp;
        st->samp_cap = kit.samp_cap;
    } else {
        TRY(cudaStreamCreateWithFlags(&st->stream, cudaStreamNonBlocking));
    }
    e = cudaMalloc(&st->re, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&st->im, bytes);
    if (e != cudaSuccess) {
        fail(ZC_ERR_MEMORY, std::string("device allocation of the state failed: ") + cudaGetErrorString(e));
        cudaGetLastError();
        zc_destroy(st);
        return ZC_ERR_MEMORY;
    }
    if (!st->arena.host) {
        TRY(cudaMallocHost(&st->arena.host, kArenaBytes));
        TRY(cudaMalloc(&st->arena.dev, kArenaBytes));
        st->arena.cap = kArenaBytes;
        TRY(cudaMalloc(&st->d_scalar, sizeof(double)));
        TRY(cudaMalloc(&st->d_err, kErrWords * sizeof(int)));
        TRY(cudaMallocHost(&st->h_scalar, sizeof(double)));
    }
    TRY(cudaMemsetAsync(st->d_err, 0, kErrWords * sizeof(int), st->stream));
#undef TRY
    rc = launch_reset(st);
    if (rc) {
        zc_destroy(st);
        return rc;
    }
    *out = st;
    return ZC_OK;
}

extern "C" {

void zc_destroy(zc_state *st) {
    if (!st) return;
    const bool healthy = !st->stream || cudaStreamSynchronize(st->stream) == cudaSuccess;
    if (st->re) cudaFree(st->re);
    if (st->im) cudaFree(st->im);
    for (auto &r : st->prof_recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : st->prof_pool) cudaEventDestroy(e);
    Kit kit;
    kit.device = st->device;
    kit.stream = st->stream;
    kit.arena = st->arena;
    kit.d_scalar = st->d_scalar;
    kit.h_scalar = st->h_scalar;
    kit.d_err = st->d_err;
    kit.d_part = st->d_part;
    kit.part_cap = st->part_cap;
    kit.d_samp = st->d_samp;
    kit.samp_cap = st->samp_cap;
    // a complete kit from a state whose stream finished cleanly goes back to the cache
    const bool complete = kit.stream && kit.arena.host && kit.arena.dev && kit.d_scalar && kit.h_scalar && kit.d_err;
    if (!(healthy && complete && give_kit(kit))) free_kit(kit);
    delete st;
}

const char *zc_name(const zc_state *st) { return st ? st->name.c_str() : ""; }

int zc_apply_unitary(zc_state *st, const uint32_t *qs, uint32_t k, const double *mat) {
    int rc = check_support(st, qs, k, kMaxUnitaryQubits, "apply_unitary");
    if (rc) return rc;
    if (!mat) return fail(ZC_ERR_INVALID, "apply_unitary: null matrix");
    QOp op{Q_UNITARY, k, {}, 0, 0, std::vector<double>(mat, mat + 2 * ((size_t)1 << (2 * k)))};
    for (uint32_t i = 0; i < k; i++) op.qs[i] = qs[i];
    return enqueue(st, std::move(op));
}

int zc_apply_diagonal(zc_state *st, const uint32_t *qs, uint32_t k, const double *d) {
    int rc = check_support(st, qs, k, kMaxDiagQubits, "apply_diagonal");
    if (rc) return rc;
    if (!d) return fail(ZC_ERR_INVALID, "apply_diagonal: null diagonal");
    QOp op{Q_DIAG, k, {}, 0, 0, std::vector<double>(d, d + 2 * ((size_t)1 << k))};
    for (uint32_t i = 0; i < k; i++) op.qs[i] = qs[i];
    return enqueue(st, std::move(op));
}

int zc_apply_cx(zc_state *st, uint32_t c, uint32_t t) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    if (c >= st->n || t >= st->n || c == t) return fail(ZC_ERR_INVALID, "apply_cx: bad control/target");
    return enqueue(st, QOp{Q_CX, 0, {}, c, t, {}});
}

int zc_apply_swap(zc_state *st, uint32_t a, uint32_t b) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    if (a >= st->n || b >= st->n || a == b) return fail(ZC_ERR_INVALID, "apply_swap: bad qubits");
    return enqueue(st, QOp{Q_SWAP, 0, {}, std::min(a, b), std::max(a, b), {}});
}

int zc_prob_one(zc_state *st, uint32_t q, double *out) {
    if (!st || !out) return fail(ZC_ERR_INVALID, "null argument");
    if (q >= st->n) return fail(ZC_ERR_INVALID, "prob_one: qubit out of range");
    int rc = flush(st);
    if (rc) return rc;
    size_t nch = 0;
    rc = launch_chunk_sums(st, 1, q, &nch, exact(st));
    if (rc) return rc;
    rc = launch_serial_sum(st, nch, exact(st));
    if (rc) return rc;
    return sync_read_scalar(st, out);
}

int zc_measure(zc_state *st, uint32_t q, double u, int *outcome) {
    if (!outcome) return fail(ZC_ERR_INVALID, "null argument");
    double p1 = 0.0;
    int rc = zc_prob_one(st, q, &p1);
    if (rc) return rc;
    const int o = u < p1;
    const double p = o ? p1 : 1.0 - p1;
    rc = launch_collapse(st, q, o, 1.0 / sqrt(p));
    if (rc) return rc;
    *outcome = o;
    return ZC_OK;
}

int zc_reset_all(zc_state *st) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    st->queue.clear();  // queued ops act on a state that is being discarded
    return launch_reset(st);
}

int zc_norm_sqr(zc_state *st, double *out) {
    if (!st || !out) return fail(ZC_ERR_INVALID, "null argument");
    int rc = flush(st);
    if (rc) return rc;
    size_t nch = 0;
    rc = launch_chunk_sums(st, 0, 0, &nch, exact(st));
    if (rc) return rc;
    rc = launch_serial_sum(st, nch, exact(st));
    if (rc) return rc;
    return sync_read_scalar(st, out);
}

// Backend::sample: pass 1 (chunk masses) and pass 2 (per-chunk rescans) run
// on the GPU, the routing between them on the host.
int zc_sample(zc_state *st, uint64_t shots, uint64_t seed, uint64_t *out) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    if (shots == 0) return ZC_OK;
    if (!out) return fail(ZC_ERR_INVALID, "sample: null output");
    int rc = flush(st);
    if (rc) return rc;
    size_t nch = 0;
    rc = launch_chunk_sums(st, 0, 0, &nch, exact(st));
    if (rc) return rc;
    std::vector<double> sums(nch);
    ZC_CUDA(cudaMemcpyAsync(sums.data(), st->d_part, nch * sizeof(double), cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    SampleRoute route;
    sample_route(sums.data(), nch, st->len, shots, seed, &route);
    rc = grow(&st->d_samp, &st->samp_cap, sample_pass2_bytes(st, route));
    if (rc) return rc;
    uint64_t *d_out = nullptr;
    rc = sample_launch_pass2(st, route, (char *)st->d_samp, &d_out);
    if (rc) return rc;
    ZC_CUDA(cudaMemcpyAsync(out, d_out, shots * sizeof(uint64_t), cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    return check_device_error(st);
}

int zc_statevector(zc_state *st, double *out) {
    if (!st || !out) return fail(ZC_ERR_INVALID, "null argument");
    int rc = flush(st);
    if (rc) return rc;
    const size_t es = st->prec / 8;
    std::vector<char> re(st->len * es), im(st->len * es);
    ZC_CUDA(cudaMemcpyAsync(re.data(), st->re, st->len * es, cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaMemcpyAsync(im.data(), st->im, st->len * es, cudaMemcpyDeviceToHost, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    if ((rc = check_device_error(st))) return rc;
    for (size_t i = 0; i < st->len; i++) {
        if (st->prec == 64) {
            out[2 * i] = ((double *)re.data())[i];
            out[2 * i + 1] = ((double *)im.data())[i];
        } else {
            out[2 * i] = (double)((float *)re.data())[i];
            out[2 * i + 1] = (double)((float *)im.data())[i];
        }
    }
    return ZC_OK;
}

int zc_load_state(zc_state *st, const double *in) {
    if (!st || !in) return fail(ZC_ERR_INVALID, "null argument");
    st->queue.clear();
    const size_t es = st->prec / 8;
    std::vector<char> re(st->len * es), im(st->len * es);
    for (size_t i = 0; i < st->len; i++) {
        if (st->prec == 64) {
            ((double *)re.data())[i] = in[2 * i];
            ((double *)im.data())[i] = in[2 * i + 1];
        } else {
            ((float *)re.data())[i] = (float)in[2 * i];
            ((float *)im.data())[i] = (float)in[2 * i + 1];
        }
    }
    ZC_CUDA(cudaMemcpyAsync(st->re, re.data(), st->len * es, cudaMemcpyHostToDevice, st->stream));
    ZC_CUDA(cudaMemcpyAsync(st->im, im.data(), st->len * es, cudaMemcpyHostToDevice, st->stream));
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    return ZC_OK;
}

int zc_finish(zc_state *st) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    int rc = flush(st);
    if (rc) return rc;
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    ZC_CUDA(cudaGetLastError());
    return check_device_error(st);
}

int zc_get_stream(zc_state *st, void **stream) {
    if (!st || !stream) return fail(ZC_ERR_INVALID, "null argument");
    *stream = (void *)st->stream;
    return ZC_OK;
}

int zc_profile(zc_state *st, int enable) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    for (auto &r : st->prof_recs) {
        st->prof_pool.push_back(r.a);
        st->prof_pool.push_back(r.b);
    }
    st->prof_recs.clear();
    st->prof = enable != 0;
    return ZC_OK;
}

int zc_profile_read(zc_state *st, zc_kernel_stat *out, int cap, int *n) {
    if (!st || !n) return fail(ZC_ERR_INVALID, "null argument");
    int rc = flush(st);
    if (rc) return rc;
    ZC_CUDA(cudaStreamSynchronize(st->stream));
    zc_kernel_stat agg[K_NKINDS];
    memset(agg, 0, sizeof agg);
    for (const auto &r : st->prof_recs) {
        float ms = 0.f;
        ZC_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        agg[r.kind].launches++;
        agg[r.kind].ms += ms;
        agg[r.kind].bytes += r.bytes;
    }
    int m = 0;
    for (int k = 0; k < K_NKINDS; k++) {
        if (!agg[k].launches) continue;
        if (m < cap && out) {
            out[m] = agg[k];
            snprintf(out[m].name, sizeof out[m].name, "%s", kKernelNames[k]);
        }
        m++;
    }
    *n = m;
    return ZC_OK;
}

int zc_set_sweep_shape(zc_state *st, uint32_t max_high) {
    if (!st) return fail(ZC_ERR_INVALID, "null state");
    if (max_high > kMaxSweepHigh) return fail(ZC_ERR_INVALID, "sweep shape: at most 7 high qubits per tile");
    int rc = flush(st);  // queued ops keep the shape they were planned for
    if (rc) return rc;
    st->sweep_high = max_high;
    return ZC_OK;
}

int zc_get_counters(zc_state *st, zc_counters *out) {
    if (!st || !out) return fail(ZC_ERR_INVALID, "null argument");
    *out = st->ctr;
    return ZC_OK;
}

}  // extern "C"
