// Internal declarations shared by the CUDA translation units of libzeno_cuda.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/zeno_cuda.h"

namespace zc {

// Sets the thread-local error text and returns `code`.
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *where);

#define ZC_CUDA(call)                                   \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return zc::cuda_fail(e_, #call); \
    } while (0)

constexpr int kMaxUnitaryQubits = 7;
constexpr int kMaxDiagQubits = 12;
constexpr int kSampleChunkLog2 = 16;  // sample.rs CHUNK = 1 << 16
constexpr int kErrWords = 16;         // device error record (d_err) in ints

// Device parameter arena: tables (matrices, diagonals) for queued ops are
// staged in pinned host memory and copied into a device ring. Wrapping the
// ring synchronises the stream, so no slot is reused while in flight.
struct Arena {
    char *host = nullptr;
    char *dev = nullptr;
    size_t cap = 0;
    size_t head = 0;
};

struct Launch {
    int blocks;
    int threads;
};

// Kernel classes for the per-launch profiler (zc_profile / zc_profile_read).
enum : int {
    K_1Q = 0, K_KQ, K_DIAG1, K_DIAGK, K_CX, K_SWAP, K_SWEEP, K_CHUNK_SUMS, K_SERIAL_SUM, K_SAMPLE_SCAN,
    K_COLLAPSE, K_RESET, K_TRAJ, K_TC, K_NKINDS
};
extern const char *const kKernelNames[K_NKINDS];

struct ProfRec {
    int kind;
    double bytes;
    cudaEvent_t a, b;
};

// An op accepted by the ABI and not yet launched.
enum : int { Q_UNITARY = 0, Q_DIAG = 1, Q_CX = 2, Q_SWAP = 3 };
struct QOp {
    int kind;
    uint32_t k;
    uint32_t qs[12];  // sorted support (unitary / diagonal)
    uint32_t a, b;    // CX control/target, SWAP qubits
    std::vector<double> data;  // interleaved c64 table
};

}  // namespace zc

struct zc_state {
    uint32_t n = 0;
    int prec = 64;  // 32 or 64
    uint32_t flags = 0;
    uint32_t sweep_high = 0;  // high (non-row) qubits per sweep tile; 0 = automatic
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    void *re = nullptr;  // device, 2^n elements of T
    void *im = nullptr;
    size_t len = 0;
    zc::Arena arena;
    // scratch for reductions and the sampler
    double *d_part = nullptr;  // chunk partial sums
    size_t part_cap = 0;
    double *d_scalar = nullptr;  // single result
    double *h_scalar = nullptr;  // pinned
    void *d_samp = nullptr;      // sampler work area
    size_t samp_cap = 0;
    int *d_err = nullptr;        // device error flag (sweep wait timeouts)
    bool df_resident = false;    // inside a flush: fast f64 sweeps left packed float pairs in re / im
    std::vector<zc::QOp> queue;  // ops waiting to be scheduled into sweeps
    bool prof = false;            // record CUDA events around every launch
    std::vector<zc::ProfRec> prof_recs;
    std::vector<cudaEvent_t> prof_pool;
    zc_counters ctr{};
    std::string name;
};

namespace zc {

// Kernel launchers (zc_gates.cu / zc_reduce.cu). All are asynchronous on
// st->stream and return ZC_OK or an error code.
// Records CUDA events around one launch on st->stream while profiling is on.
struct ProfScope {
    zc_state *st;
    long idx = -1;
    ProfScope(zc_state *s, int kind, double bytes);
    ~ProfScope();
};

// Reads the state's device error record after a sync (a kernel that gave
// up on a bounded wait or found an index out of range): ZC_ERR_CUDA with
// the record's text, and the record cleared; else ZC_OK.
int check_device_error(zc_state *st);
// mem::plan against `budget` bytes (ZC_ERR_MEMORY with zeno's text), and
// zc_create_ex with that budget in place of 0.75 of the device memory.
int plan_state(uint32_t n, int prec, uint64_t budget);
int create_state(uint32_t n, int prec, uint32_t flags, uint64_t budget, zc_state **out);

int launch_1q(zc_state *st, uint32_t q, const double *m8, bool exact);
int launch_kq(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_mat, bool exact);
// Dense k-qubit block (k = 2..7) on an f64 state in fast mode, double-float
// on the FP32 pipe; dev_mat_df: row-major 2^k x 2^k float4 (re hi, re lo,
// im hi, im lo) per entry.
int launch_kq_df(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_mat_df);
// Dense k-qubit block (k = 3..7) on tensor cores, f32 state, 3xTF32 (zc_tc.cu);
// mat: row-major 2^k x 2^k complex (interleaved f64 pairs).
int launch_block_tc(zc_state *st, const uint32_t *qs, uint32_t k, const double *mat);
int launch_diag1(zc_state *st, uint32_t q, const double *d4, bool exact);
int launch_diagk(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_diag, bool exact);
int launch_cx(zc_state *st, uint32_t c, uint32_t t);
int launch_swap(zc_state *st, uint32_t a, uint32_t b);
int launch_reset(zc_state *st);
int launch_collapse(zc_state *st, uint32_t q, int outcome, double scale64);
// f64 partial sums of |amp|^2 over chunks of 2^16 (exact: serial within a
// chunk in the reference's order; otherwise parallel double-float).
// mode 0: all amplitudes (norm / sampler pass 1); mode 1: the q=1 half of
// qubit q (prob_one). Writes nchunks partials to `out` (default st->d_part).
int launch_chunk_sums(zc_state *st, int mode, uint32_t q, size_t *nchunks, bool exact, double *out = nullptr);
// Sum of st->d_part[0..nchunks) into st->d_scalar (exact: serial, in order).
int launch_serial_sum(zc_state *st, size_t nchunks, bool exact);
// Sampler pass 2 (sample.rs:64-108): a touched chunk and its draws.
struct SampleChunk {
    uint64_t chunk;  // chunk index
    uint64_t s0, s1; // draw range
    double cum;      // cum_before[chunk]
};
}  // namespace zc
#include "zc_sweep.h"
namespace zc {
// A planned sweep: tile geometry, encoded micro-ops, diagonal tables and the
// queue indices it consumes.
struct SweepPlan {
    SweepGeom g;
    std::vector<MicroOp> mops;
    std::vector<char> tables;
    std::vector<size_t> taken;
    std::vector<QOp> carry;  // diagonals left pending by the sweep: they go to the queue front
};
size_t plan_sweep(uint32_t n, int prec, bool ex, uint32_t L, uint32_t Hcap, const std::vector<QOp> &q,
                  SweepPlan *plan);
void erase_taken(std::vector<QOp> &q, const std::vector<size_t> &taken);
// Remove the plan's ops from the queue and put its carried diagonals in front.
void consume_plan(std::vector<QOp> &q, SweepPlan &plan);

// A sweep op in global qubits before encoding (kind: MOP_*). DK: ascending
// support `sup` and an interleaved complex table over it.
struct LoweredOp {
    uint32_t kind = 0;
    uint32_t a = 0, b = 0;
    double m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    std::vector<uint32_t> sup;
    std::vector<double> tab;
};
// Double-float lowering of a fast f64 sweep: one-qubit gates as diagonal *
// real * diagonal, the diagonals propagated and merged into table ops placed
// before the register runs of at most run_cap gates. Pending diagonals at the
// end go to *carry (when it is given and the sequence has a non-diagonal op).
void lower_df(const std::vector<const QOp *> &seq, int run_cap, std::vector<LoweredOp> *out,
              std::vector<QOp> *carry);
int launch_single(zc_state *st, const QOp &op);
int launch_sweep_multi(cudaStream_t stream, int num_sms, int prec, bool exact, const char *dev_blob, int *d_err);
int arena_put(zc_state *st, const void *src, size_t bytes, const void **dev);
// Round an f64 state left as double-float pairs (g.form kFormOutDf) back to f64.
int launch_df_to_f64(zc_state *st);
int launch_sweep(zc_state *st, const SweepGeom &g, const MicroOp *dev_ops, int nops, const char *dev_tables,
                 bool exact);
struct TrajOp;
struct TrajNoise;
int launch_trajectories(zc_state *st, uint32_t n, const TrajOp *d_ops, int nops, const double *d_mats,
                        const uint32_t *d_fq, const uint32_t *d_fc, int nfinal, const TrajNoise &nz, uint64_t ntraj,
                        uint64_t seed, uint64_t *d_out, void *d_work, int ctas);
// d_scratch: sample_scan_scratch(nchunks, chunk_len, exact) bytes of device memory.
int launch_sample_scan(zc_state *st, const SampleChunk *d_chunks, size_t nchunks, const double *d_us,
                       uint64_t *d_out, uint64_t chunk_len, bool exact, void *d_scratch);
size_t sample_scan_scratch(size_t nchunks, uint64_t chunk_len, bool exact);
// Sampler phases, so a caller can sample many states with two syncs.
struct SampleRoute {
    std::vector<double> us;            // sorted scaled draws
    std::vector<SampleChunk> touched;  // chunks that received draws
    uint64_t chunk_len = 0;
};
void sample_route(const double *sums, size_t nch, uint64_t len, uint64_t shots, uint64_t seed, SampleRoute *r);
size_t sample_pass2_bytes(const zc_state *st, const SampleRoute &r);
int sample_launch_pass2(zc_state *st, const SampleRoute &r, char *d_work, uint64_t **d_out);

}  // namespace zc
