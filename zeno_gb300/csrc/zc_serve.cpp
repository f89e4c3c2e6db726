// Continuous-batching serving engine.
//
// zeno runs one circuit per call (src/lib.rs:248, src/exec.rs:407-452).
// A server keeps many circuits' states resident in one HBM pool and
// advances all of them together:
//   * submit  — a compiled static program joins a FIFO of pending requests;
//   * step    — pending requests are admitted while their state fits the pool
//               and a slot is free (admission by HBM footprint); every active
//               request contributes its next sweep (planned exactly like a
//               lone state's) to ONE packed launch over all states, replayed
//               from a captured CUDA graph; ops that do not fit a sweep
//               (dense k>=2 blocks) run on their own; requests whose op queue
//               is empty are sampled (the same sampler and seed semantics as a
//               lone run) and their slots are freed for the next admissions;
//   * take    — the caller collects a finished request's sampled indices.
// Requests that arrive while others are on the GPU are admitted at the next
// step, so their work overlaps on the device with the requests in flight.
// In exact mode a request's result is bit-identical to running it alone.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <map>
#include <vector>

#include "zc_internal.h"
#include "zc_pool.h"
#include "zc_rng.h"
#include "../../include/zeno_cuda_serve.h"
#include "zc_sweep.h"

namespace zc {
namespace {

constexpr uint64_t kServeMaxShots = 65536;
constexpr uint32_t kServeMaxQubits = 30;
constexpr size_t kBlobBytes = 16u << 20;
constexpr int kRounds = 4;  // packed launches per precision per step (one host blob each)

struct Request {
    uint64_t id = 0;
    uint32_t n = 0;
    int prec = 32;
    uint64_t shots = 0, seed = 0;
    std::vector<QOp> queue;
    std::vector<std::pair<uint32_t, uint32_t>> finals;
    size_t off = 0, bytes = 0;
    zc_state view;  // re/im in the pool; stream and scratch borrowed from the server
    std::vector<uint64_t> result;
};

struct Group {  // one precision: its packed-launch graph and blob buffers
    char *h_blob[kRounds] = {};
    char *d_blob = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t copy_node = nullptr;
    uint64_t launches = 0;
};

}  // namespace
}  // namespace zc

struct zc_server {
    zc_state *ctx = nullptr;  // stream, parameter arena, reduction scratch, error flag
    char *pool = nullptr;
    size_t pool_bytes = 0;
    zc::PoolFreeList free_list;  // offsets of the pool not held by active requests
    uint32_t max_slots = 0;
    uint32_t flags = 0;
    uint64_t next_id = 1;
    std::deque<zc::Request *> pending;
    std::vector<zc::Request *> active;
    std::map<uint64_t, zc::Request *> done;
    zc::Group groups[2];  // [0] f32, [1] f64
    // batched sampling of a step's finished requests
    double *d_bpart = nullptr, *h_bpart = nullptr;
    size_t bpart_cap = 0, hbpart_cap = 0;
    char *d_bwork = nullptr;
    size_t bwork_cap = 0;
    uint64_t *h_bout = nullptr;
    size_t hbout_cap = 0;
    uint64_t launches = 0, packed_launches = 0, admitted = 0, completed = 0;
    uint64_t steps = 0, plan_us = 0, sample_us = 0, wait_us = 0;
    double device_ms = 0.0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace zc {
namespace {

// A state view over pool memory that borrows the server context's stream
// and parameter ring.
void make_view(zc_server *s, Request *r) {
    zc_state &v = r->view;
    const zc_state *c = s->ctx;
    v.n = r->n;
    v.prec = r->prec;
    v.flags = s->flags | ZC_FLAG_NO_SWEEPS;  // ops reach it only through the server's planner
    v.device = c->device;
    v.num_sms = c->num_sms;
    v.stream = c->stream;
    v.len = 1ull << r->n;
    const size_t half = v.len * (r->prec / 8);
    v.re = s->pool + r->off;
    v.im = s->pool + r->off + half;
    v.arena = c->arena;
    v.d_part = nullptr;  // the server samples with its own batch buffers
    v.part_cap = 0;
    v.d_scalar = c->d_scalar;
    v.h_scalar = c->h_scalar;
    v.d_samp = nullptr;
    v.samp_cap = 0;
    v.d_err = c->d_err;
    v.name = r->prec == 64 ? "cuda-f64" : "cuda-f32";
}

uint64_t tile_shape(const Request *r, uint32_t *L, uint32_t *Hcap) {
    *L = std::min<uint32_t>(r->n, r->prec == 64 ? 5 : 6);
    const uint32_t Tmax = r->prec == 64 ? 12 : 13;
    *Hcap = std::min<uint32_t>(std::min<uint32_t>(Tmax - *L, r->n - *L), kMaxSweepHigh);
    return 0;
}

int capture_group(zc_server *s, int gi) {
    Group &g = s->groups[gi];
    cudaStream_t st = s->ctx->stream;
    ZC_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaMemcpyAsync(g.d_blob, g.h_blob[0], sizeof(SweepBatch), cudaMemcpyHostToDevice, st);
    int rc = launch_sweep_multi(st, s->ctx->num_sms, gi ? 64 : 32, (s->flags & ZC_FLAG_FAST) == 0, g.d_blob,
                                s->ctx->d_err);
    cudaError_t e = cudaStreamEndCapture(st, &g.graph);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    size_t n = 0;
    ZC_CUDA(cudaGraphGetNodes(g.graph, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    ZC_CUDA(cudaGraphGetNodes(g.graph, nodes.data(), &n));
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        ZC_CUDA(cudaGraphNodeGetType(nd, &t));
        if (t == cudaGraphNodeTypeMemcpy) g.copy_node = nd;
    }
    if (!g.copy_node) return fail(ZC_ERR_CUDA, "packed launch graph has no copy node");
    ZC_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
    return ZC_OK;
}

// Build and launch the packed sweep of every active request of one precision
// (round `round` of the step: its host blob stays untouched until the step's
// final sync). *issued counts the launches made.
int packed_step(zc_server *s, int gi, int round, int *issued) {
    Group &g = s->groups[gi];
    const int prec = gi ? 64 : 32;
    const bool ex = (s->flags & ZC_FLAG_FAST) == 0;
    std::vector<SweepJob> jobs;
    std::vector<char> body;  // micro-ops + tables, offsets relative to the body
    std::vector<std::pair<Request *, SweepPlan>> planned;
    uint64_t tiles = 0;
    for (Request *r : s->active) {
        if (r->prec != prec || r->queue.empty()) continue;
        uint32_t L, Hcap;
        tile_shape(r, &L, &Hcap);
        SweepPlan plan;
        if (plan_sweep(r->n, r->prec, ex, L, Hcap, r->queue, &plan) <= 1) {
            // the front op runs on its own (a dense k >= 2 block, or nothing to batch);
            // the view shares the server's parameter ring
            r->view.arena = s->ctx->arena;
            int rc = launch_single(&r->view, r->queue.front());
            s->ctx->arena = r->view.arena;
            if (rc) return rc;
            r->queue.erase(r->queue.begin());
            s->launches++;
            (*issued)++;
            continue;
        }
        SweepJob j{};
        j.re = r->view.re;
        j.im = r->view.im;
        j.L = plan.g.L;
        j.H = plan.g.H;
        j.nops = (uint32_t)plan.mops.size();
        for (uint32_t k = 0; k < plan.g.H && k < 8; k++) j.hpos[k] = plan.g.hpos[k];
        j.ntiles = plan.g.ntiles;
        j.tile_start = tiles;
        tiles += plan.g.ntiles;
        size_t off = (body.size() + 15) & ~(size_t)15;
        body.resize(off + plan.mops.size() * sizeof(MicroOp));
        memcpy(body.data() + off, plan.mops.data(), plan.mops.size() * sizeof(MicroOp));
        j.ops_off = off;
        off = (body.size() + 15) & ~(size_t)15;
        body.resize(off + plan.tables.size());
        if (!plan.tables.empty()) memcpy(body.data() + off, plan.tables.data(), plan.tables.size());
        j.tables_off = off;
        jobs.push_back(j);
        planned.push_back({r, std::move(plan)});
    }
    if (jobs.empty()) return ZC_OK;
    const size_t head = sizeof(SweepBatch) + jobs.size() * sizeof(SweepJob);
    const size_t body_off = (head + 255) & ~(size_t)255;
    const size_t total = body_off + body.size();
    if (total > kBlobBytes) return fail(ZC_ERR_INVALID, "packed launch exceeds its parameter buffer");
    for (auto &j : jobs) {
        j.ops_off += body_off;
        j.tables_off += body_off;
    }
    SweepBatch hdr{(uint32_t)jobs.size(), 0, tiles};
    char *hb = g.h_blob[round];
    memcpy(hb, &hdr, sizeof hdr);
    memcpy(hb + sizeof hdr, jobs.data(), jobs.size() * sizeof(SweepJob));
    memcpy(hb + body_off, body.data(), body.size());
    if (!g.exec && g.graph == nullptr && g.launches > 0) {
        int rc = capture_group(s, gi);
        if (rc) return rc;
    }
    if (g.exec) {
        ZC_CUDA(cudaGraphExecMemcpyNodeSetParams1D(g.exec, g.copy_node, g.d_blob, hb, total, cudaMemcpyHostToDevice));
        ZC_CUDA(cudaGraphLaunch(g.exec, s->ctx->stream));
    } else {
        // first packed launch of the server runs uncaptured (kernel attributes get set here)
        ZC_CUDA(cudaMemcpyAsync(g.d_blob, hb, total, cudaMemcpyHostToDevice, s->ctx->stream));
        int rc = launch_sweep_multi(s->ctx->stream, s->ctx->num_sms, prec, ex, g.d_blob, s->ctx->d_err);
        if (rc) return rc;
    }
    s->launches++;
    s->packed_launches++;
    g.launches++;
    (*issued)++;
    for (auto &pr : planned) consume_plan(pr.first->queue, pr.second);
    return ZC_OK;
}

// Grow a device or pinned host buffer to at least `need` bytes (contents dropped).
int grow_dev(void **p, size_t *cap, size_t need) {
    if (need <= *cap) return ZC_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    ZC_CUDA(cudaMalloc(p, need));
    *cap = need;
    return ZC_OK;
}
int grow_host(void **p, size_t *cap, size_t need) {
    if (need <= *cap) return ZC_OK;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    ZC_CUDA(cudaMallocHost(p, need));
    *cap = need;
    return ZC_OK;
}

// Sample every finished request of a step with two device syncs in total:
// all chunk-mass passes, one copy back; host routing per request; all
// rescans, one copy of every index list back. Per request this is exactly
// zc_sample (same kernels, same order, same seed stream).
int sample_finished(zc_server *s, const std::vector<Request *> &fin) {
    zc_state *c = s->ctx;
    const bool ex = (s->flags & ZC_FLAG_FAST) == 0;
    std::vector<size_t> part_off(fin.size()), nch(fin.size());
    size_t tot_ch = 0;
    for (size_t i = 0; i < fin.size(); i++) {
        const uint64_t len = 1ull << fin[i]->n;
        const uint64_t chunk = len < (1ull << kSampleChunkLog2) ? len : (1ull << kSampleChunkLog2);
        nch[i] = (size_t)((len + chunk - 1) / chunk);
        part_off[i] = tot_ch;
        tot_ch += nch[i];
    }
    if (tot_ch == 0) return ZC_OK;
    int rc = grow_dev((void **)&s->d_bpart, &s->bpart_cap, tot_ch * sizeof(double));
    if (rc == ZC_OK) rc = grow_host((void **)&s->h_bpart, &s->hbpart_cap, tot_ch * sizeof(double));
    if (rc) return rc;
    for (size_t i = 0; i < fin.size(); i++) {
        size_t n = 0;
        if ((rc = launch_chunk_sums(&fin[i]->view, 0, 0, &n, ex, s->d_bpart + part_off[i]))) return rc;
    }
    ZC_CUDA(cudaMemcpyAsync(s->h_bpart, s->d_bpart, tot_ch * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ZC_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<SampleRoute> routes(fin.size());
    std::vector<size_t> work_off(fin.size()), out_off(fin.size());
    size_t tot_work = 0, tot_out = 0;
    for (size_t i = 0; i < fin.size(); i++) {
        Request *r = fin[i];
        sample_route(s->h_bpart + part_off[i], nch[i], 1ull << r->n, r->shots, splitmix64(r->seed), &routes[i]);
        work_off[i] = tot_work;
        tot_work += (sample_pass2_bytes(&r->view, routes[i]) + 255) & ~(size_t)255;
        out_off[i] = tot_out;
        tot_out += r->shots;
    }
    if ((rc = grow_dev((void **)&s->d_bwork, &s->bwork_cap, tot_work))) return rc;
    if ((rc = grow_host((void **)&s->h_bout, &s->hbout_cap, tot_out * sizeof(uint64_t)))) return rc;
    for (size_t i = 0; i < fin.size(); i++) {
        Request *r = fin[i];
        uint64_t *d_out = nullptr;
        r->view.arena = c->arena;  // the view shares the server's parameter ring
        rc = sample_launch_pass2(&r->view, routes[i], s->d_bwork + work_off[i], &d_out);
        c->arena = r->view.arena;
        if (rc) return rc;
        ZC_CUDA(cudaMemcpyAsync(s->h_bout + out_off[i], d_out, r->shots * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                                c->stream));
    }
    ZC_CUDA(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < fin.size(); i++)
        fin[i]->result.assign(s->h_bout + out_off[i], s->h_bout + out_off[i] + fin[i]->shots);
    return ZC_OK;
}

QOp to_qop(const zc_op_view &v) {
    QOp q{};
    q.kind = v.kind == ZC_OP_UNITARY ? Q_UNITARY : v.kind == ZC_OP_DIAG ? Q_DIAG : v.kind == ZC_OP_CX ? Q_CX : Q_SWAP;
    q.k = v.k;
    for (uint32_t i = 0; i < v.k && i < 12; i++) q.qs[i] = v.qubits[i];
    q.a = v.a;
    q.b = v.b;
    if (v.data) {
        const size_t cnt = v.kind == ZC_OP_UNITARY ? ((size_t)1 << (2 * v.k)) : ((size_t)1 << v.k);
        q.data.assign(v.data, v.data + 2 * cnt);
    }
    return q;
}

}  // namespace
}  // namespace zc

using namespace zc;

extern "C" {

int zc_server_create(const zc_server_options *opt, zc_server **out) {
    if (!opt || !out) return fail(ZC_ERR_INVALID, "null argument");
    *out = nullptr;
    zc_server *s = new zc_server();
    s->flags = opt->flags & ZC_FLAG_FAST;
    s->max_slots = opt->max_slots ? opt->max_slots : 1024;
    int rc = zc_create_ex(1, 64, ZC_FLAG_NO_SWEEPS, &s->ctx);
    if (rc) {
        delete s;
        return rc;
    }
    auto bail = [&](int code) {
        zc_server_destroy(s);
        return code;
    };
    uint64_t budget = 0;
    if ((rc = zc_device_budget(0.75, &budget))) return bail(rc);
    s->pool_bytes = opt->pool_bytes ? opt->pool_bytes : budget / 2;
    cudaError_t e = cudaMalloc(&s->pool, s->pool_bytes);
    if (e != cudaSuccess) return bail(fail(ZC_ERR_MEMORY, "server pool allocation failed"));
    s->free_list.reset(s->pool_bytes);
    for (auto &g : s->groups) {
        for (auto &hb : g.h_blob)
            if ((e = cudaMallocHost(&hb, kBlobBytes)) != cudaSuccess) return bail(cuda_fail(e, "cudaMallocHost"));
        if ((e = cudaMalloc(&g.d_blob, kBlobBytes)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc"));
    }
    if ((e = cudaEventCreate(&s->ev0)) != cudaSuccess || (e = cudaEventCreate(&s->ev1)) != cudaSuccess)
        return bail(cuda_fail(e, "cudaEventCreate"));
    *out = s;
    return ZC_OK;
}

void zc_server_destroy(zc_server *s) {
    if (!s) return;
    if (s->ctx) cudaStreamSynchronize(s->ctx->stream);
    for (Request *r : s->pending) delete r;
    for (Request *r : s->active) delete r;
    for (auto &kv : s->done) delete kv.second;
    for (auto &g : s->groups) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.graph) cudaGraphDestroy(g.graph);
        for (auto hb : g.h_blob)
            if (hb) cudaFreeHost(hb);
        if (g.d_blob) cudaFree(g.d_blob);
    }
    if (s->d_bpart) cudaFree(s->d_bpart);
    if (s->h_bpart) cudaFreeHost(s->h_bpart);
    if (s->d_bwork) cudaFree(s->d_bwork);
    if (s->h_bout) cudaFreeHost(s->h_bout);
    if (s->pool) cudaFree(s->pool);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    zc_destroy(s->ctx);
    delete s;
}

int zc_server_submit(zc_server *s, const zc_program *p, int prec, uint64_t shots, uint64_t seed, uint64_t *id) {
    if (!s || !p || !id) return fail(ZC_ERR_INVALID, "null argument");
    zc_program_info info;
    int rc = zc_program_get_info(p, &info);
    if (rc) return rc;
    if (info.dynamic) return fail(ZC_ERR_UNSUPPORTED, "serve: dynamic programs run through zc_run");
    if (prec != 32 && prec != 64) return fail(ZC_ERR_INVALID, "serve: precision_bits must be 32 or 64");
    if (info.n_qubits > kServeMaxQubits) return fail(ZC_ERR_INVALID, "serve: at most 30 qubits per request");
    if (shots > kServeMaxShots) return fail(ZC_ERR_INVALID, "serve: at most 65536 shots per request");
    const size_t bytes = (((size_t)2 << info.n_qubits) * (prec / 8) + 255) & ~(size_t)255;
    if (bytes > s->pool_bytes) return fail(ZC_ERR_MEMORY, "serve: state larger than the server pool");
    Request *r = new Request();
    r->id = s->next_id++;
    r->n = info.n_qubits;
    r->prec = prec;
    r->shots = shots;
    r->seed = seed;
    r->bytes = bytes;
    for (uint64_t i = 0; i < info.nops; i++) {
        zc_op_view v;
        if ((rc = zc_program_get_op(p, i, &v))) {
            delete r;
            return rc;
        }
        r->queue.push_back(to_qop(v));
    }
    for (uint64_t i = 0; i < info.nfinal; i++) {
        uint32_t q, c;
        zc_program_get_final(p, i, &q, &c);
        r->finals.push_back({q, c});
    }
    s->pending.push_back(r);
    *id = r->id;
    return ZC_OK;
}

int zc_server_step(zc_server *s, zc_server_status *status) {
    if (!s) return fail(ZC_ERR_INVALID, "null server");
    int rc = ZC_OK;
    // 1. admission: FIFO, by HBM footprint and free slots
    while (!s->pending.empty() && s->active.size() < s->max_slots) {
        Request *r = s->pending.front();
        if (!s->free_list.alloc(r->bytes, &r->off)) break;
        s->pending.pop_front();
        make_view(s, r);
        if ((rc = launch_reset(&r->view))) return rc;
        s->active.push_back(r);
        s->admitted++;
        s->launches++;
    }
    using clk = std::chrono::steady_clock;
    auto us_since = [](clk::time_point t) {
        return (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(clk::now() - t).count();
    };
    // 2. up to kRounds packed launches per precision (plus lone launches for
    //    dense blocks), queued back to back without a host sync in between
    ZC_CUDA(cudaEventRecord(s->ev0, s->ctx->stream));
    auto t0 = clk::now();
    for (int round = 0; round < kRounds; round++) {
        int issued = 0;
        for (int gi = 0; gi < 2 && rc == ZC_OK; gi++) rc = packed_step(s, gi, round, &issued);
        if (rc) return rc;
        if (!issued) break;
    }
    s->plan_us += us_since(t0);
    // 3. completions: sample all finished requests together, free their slots
    t0 = clk::now();
    std::vector<Request *> still, fin, sampled;
    for (Request *r : s->active) {
        if (!r->queue.empty()) {
            still.push_back(r);
            continue;
        }
        fin.push_back(r);
        if (!r->finals.empty() && r->shots) sampled.push_back(r);
        else r->result.assign(r->shots, 0);
    }
    if ((rc = sample_finished(s, sampled))) return rc;
    for (Request *r : fin) {
        s->free_list.release(r->off, r->bytes);
        s->done[r->id] = r;
        s->completed++;
    }
    s->active.swap(still);
    s->sample_us += us_since(t0);
    ZC_CUDA(cudaEventRecord(s->ev1, s->ctx->stream));
    t0 = clk::now();
    ZC_CUDA(cudaStreamSynchronize(s->ctx->stream));
    s->wait_us += us_since(t0);
    float ms = 0.f;
    ZC_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->device_ms += ms;
    s->steps++;
    int h = 0;
    ZC_CUDA(cudaMemcpy(&h, s->ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) return fail(ZC_ERR_CUDA, "packed sweep gave up waiting for a bulk copy");
    if (status) {
        status->pending = s->pending.size();
        status->active = s->active.size();
        status->done = s->done.size();
        status->launches = s->launches;
        status->packed_launches = s->packed_launches;
        status->admitted = s->admitted;
        status->completed = s->completed;
        status->pool_used = s->pool_bytes - s->free_list.free_bytes();
        status->steps = s->steps;
        status->plan_us = s->plan_us;
        status->sample_us = s->sample_us;
        status->wait_us = s->wait_us;
        status->device_us = (uint64_t)(s->device_ms * 1e3);
    }
    return ZC_OK;
}

int zc_server_done_ids(zc_server *s, uint64_t *ids, size_t cap, size_t *n) {
    if (!s || !n) return fail(ZC_ERR_INVALID, "null argument");
    size_t i = 0;
    for (auto &kv : s->done) {
        if (i < cap && ids) ids[i] = kv.first;
        i++;
    }
    *n = i;
    return ZC_OK;
}

int zc_server_take(zc_server *s, uint64_t id, uint64_t *indices, uint64_t cap, uint64_t *n) {
    if (!s || !n) return fail(ZC_ERR_INVALID, "null argument");
    auto it = s->done.find(id);
    if (it == s->done.end()) return fail(ZC_ERR_INVALID, "serve: request not finished (or already taken)");
    Request *r = it->second;
    *n = r->result.size();
    for (uint64_t i = 0; i < r->result.size() && i < cap; i++) indices[i] = r->result[i];
    s->done.erase(it);
    delete r;
    return ZC_OK;
}

}  // extern "C"
