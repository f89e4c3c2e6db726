/*
 * zeno_cuda.h — C ABI of the GB300 (sm_103a) state-vector backend for zeno.
 *
 * The plain entry points mirror zeno's `exec::Backend` trait
 * (src/exec.rs:134-162) one to one, so a Rust `CudaBackend` can implement
 * the trait with a thin `extern "C"` shim. Borrowed
 * slices (`qs`, `mat`, `d`) are copied before a call returns. Complex
 * numbers cross as interleaved (re, im) doubles, the layout of
 * `num_complex::Complex<f64>`. Every call returns ZC_OK or an error code;
 * `zc_last_error()` gives the message (thread-local).
 *
 * Conventions: qubit q is bit q of a basis index (src/ir.rs:8-9); a
 * k-qubit matrix is row-major 2^k x 2^k with bit b of a local index on
 * qs[b], qs sorted ascending (src/compiler.rs:370-398).
 */
#ifndef ZENO_CUDA_H
#define ZENO_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ZC_OK 0
#define ZC_ERR_INVALID 1     /* bad argument (qubit out of range, k too large, ...) */
#define ZC_ERR_MEMORY 2      /* state does not fit the device budget, or allocation failed */
#define ZC_ERR_CUDA 3        /* CUDA runtime error (message in zc_last_error) */
#define ZC_ERR_UNSUPPORTED 4 /* no usable GPU / feature not available */

/* zc_create_ex flags */
#define ZC_FLAG_EXACT 0u      /* reference arithmetic, no FMA: bit-exact with zeno's CPU kernels */
#define ZC_FLAG_FAST 1u       /* tolerance parity, not bit-exact: f32 FMA-contracted (max |d amp| <= 1e-5
                                 vs the f64 oracle); f64 in double-float pairs on the FP32 pipe with f64
                                 storage (max |d amp| <= 1e-12) */
#define ZC_FLAG_NO_SWEEPS 2u  /* one launch per op: disables multi-op sweep scheduling */
#define ZC_FLAG_FORCE_SWEEPS 4u /* schedule sweeps even for small states (testing) */
#define ZC_FLAG_PER_SHOT 8u   /* noisy runs: replay shot by shot (zeno's order and RNG) instead of batching */
#define ZC_FLAG_TENSOR 16u    /* f32 states: dense k>=3 blocks as 3xTF32 tensor-core GEMMs (FP32 accumulation) */

typedef struct zc_state zc_state;

/* ------------------------------------------------------------------ *
 * Backend trait mirror (src/exec.rs:134-162, CpuBackend :164-225)      *
 * ------------------------------------------------------------------ */

/* exec::make_backend (src/exec.rs:306-331): allocate |0...0> with
 * precision_bits 32 or 64 on the current CUDA device. Refuses (ZC_ERR_MEMORY)
 * when the state exceeds the device budget (mem::plan, src/mem.rs:114-131). */
int zc_create(uint32_t n_qubits, int precision_bits, zc_state **out);
int zc_create_ex(uint32_t n_qubits, int precision_bits, uint32_t flags, zc_state **out);
void zc_destroy(zc_state *st);
/* Backend::name: "cuda-f64" / "cuda-f32". */
const char *zc_name(const zc_state *st);

/* Backend::apply_unitary: k in 1..=7, sorted distinct qubits, 4^k entries. */
int zc_apply_unitary(zc_state *st, const uint32_t *qs, uint32_t k, const double *mat_c64);
/* Backend::apply_diagonal: k in 1..=12, sorted distinct qubits, 2^k entries. */
int zc_apply_diagonal(zc_state *st, const uint32_t *qs, uint32_t k, const double *diag_c64);
/* Backend::apply_cx: zero-arithmetic permutation (state.rs apply_cx :397-417). */
int zc_apply_cx(zc_state *st, uint32_t control, uint32_t target);
/* SWAP as a zero-arithmetic permutation (no counterpart in the trait: zeno
 * runs SWAP as a dense 4x4 unitary, src/gates.rs:156). */
int zc_apply_swap(zc_state *st, uint32_t a, uint32_t b);
/* Backend::prob_one (state.rs prob_one :599-626), f64 accumulation. */
int zc_prob_one(zc_state *st, uint32_t q, double *out);
/* Backend::measure (exec.rs:201-207): outcome = u < P(1); collapses. */
int zc_measure(zc_state *st, uint32_t q, double u, int *outcome);
/* Backend::reset_all: back to |0...0>. */
int zc_reset_all(zc_state *st);
/* Backend::sample (exec.rs:213-216 + sample.rs:29-111): `shots` ascending
 * basis indices drawn with xoshiro256++ seeded by seed_from_u64(seed). */
int zc_sample(zc_state *st, uint64_t shots, uint64_t seed, uint64_t *out);
/* Backend::statevector: 2^n interleaved (re, im) doubles. */
int zc_statevector(zc_state *st, double *out_c64);
/* Backend::norm_sqr, f64 accumulation. */
int zc_norm_sqr(zc_state *st, double *out);
/* Backend::finish: wait for all queued GPU work. */
int zc_finish(zc_state *st);

/* Backend::sample without any allocation (no counterpart in the reference).
 * For callers that cannot let the library allocate device memory when they
 * sample: runtimes that carve all device memory into their own pool at
 * start-up, or loops that must not stall on cudaMalloc/cudaFree. It draws
 * zeno's own indices — those of zc_sample on an exact-mode state — whatever
 * arithmetic flag the state was created with (on a ZC_FLAG_FAST state,
 * zc_sample's faster sums may move a draw by one index; this call does
 * not). Its scratch is a fixed ~0.9 MiB device array that every GPU loading
 * the library keeps until exit. Limits: <= 30 qubits, <= 16384 shots;
 * larger requests get ZC_ERR_INVALID. Queued ops must be flushed first
 * (zc_finish). The call synchronises the state's stream (it routes the
 * draws on the host between its two kernels). The first call on a device
 * resolves the array's device address. All calls share the array: calls
 * that overlap (on the GPU or from several threads) race. */
int zc_sample_noalloc(zc_state *st, uint64_t shots, uint64_t seed, uint64_t *out);

/* Thread-local text of the last error. */
const char *zc_last_error(void);

/* ------------------------------------------------------------------ *
 * Capacity planning retargeted to HBM (src/mem.rs:11-131)              *
 * ------------------------------------------------------------------ */

/* Device memory a state may use: `fraction` of the device's memory
 * (mem::budget_bytes without an explicit limit, src/mem.rs:104-111). */
int zc_device_budget(double fraction, uint64_t *bytes);
/* The device's memory the budget is taken from (mem::physical_ram_bytes,
 * src/mem.rs:9-16, retargeted): ZENO_MEM_BYTES if set, pretending to be a
 * smaller device, else the total HBM. */
int zc_device_memory(uint64_t *bytes);

/* The current device, for capacity reports (zeno info, src/main.rs:1001-1082
 * with HBM in place of RAM). */
typedef struct {
    char name[64];
    uint32_t sms, cc_major, cc_minor, _pad;
    uint64_t hbm_bytes, free_bytes, l2_bytes;
} zc_device;
int zc_device_info(zc_device *out);
uint64_t zc_state_bytes(uint32_t n_qubits, int precision_bits);
uint32_t zc_max_qubits(uint64_t budget, int precision_bits);

/* ------------------------------------------------------------------ *
 * Harness helpers (tests and benchmarks)                               *
 * ------------------------------------------------------------------ */

/* Overwrite the state with 2^n interleaved (re, im) doubles. */
int zc_load_state(zc_state *st, const double *amps_c64);
/* The CUDA stream (cudaStream_t) all of this state's work runs on. */
int zc_get_stream(zc_state *st, void **stream);

typedef struct {
    uint64_t ops;            /* ops accepted */
    uint64_t launches;       /* kernels launched */
    uint64_t sweeps;         /* full-state passes issued by gate kernels */
    uint64_t bytes_moved;    /* algorithmic HBM bytes of those passes */
    uint64_t micro_ops[8];   /* ops inside multi-op sweeps, by kind: 1 complex 2x2, 2 one-qubit
                                diagonal, 3 table diagonal, 4 CX, 5 SWAP, 6 real 2x2, 7 rotation */
} zc_counters;
int zc_get_counters(zc_state *st, zc_counters *out);

/* Sweep tile shape: at most `max_high` (1..7) qubits above the 256-byte row
 * per tile; 0 restores the automatic choice. Queued ops are flushed first.
 * Used by the autotuner (zeno_gb300/autotune.py); results do not depend on it. */
int zc_set_sweep_shape(zc_state *st, uint32_t max_high);

/* Arithmetic issue rates of the current device, measured by timing
 * issue-bound FMA loops (no counterpart in the reference): the compute
 * denominators of the rooflines the benchmarks report beside HBM GB/s
 * (double-float f64 sweeps run on the FP32 pipe, exact f64 on the FP64
 * pipe). Rates are FMA operations per second over the whole device. */
typedef struct {
    double fp64_fma_per_s;
    double fp32_fma_per_s;
    uint32_t sms, _pad;
} zc_arith_peaks;
int zc_measure_arith_peaks(zc_arith_peaks *out);

/* Per-launch profiling: with profiling on, every kernel launch of this
 * state is bracketed by CUDA events on its stream. zc_profile(st, 1)
 * starts (and clears) a recording, zc_profile_read flushes, synchronises
 * and returns one entry per kernel class that ran: launches, total time
 * and the algorithmic HBM bytes those launches move. */
typedef struct {
    char name[24];
    uint64_t launches;
    double ms;
    double bytes;
} zc_kernel_stat;
int zc_profile(zc_state *st, int enable);
int zc_profile_read(zc_state *st, zc_kernel_stat *out, int cap, int *n);

/* ------------------------------------------------------------------ *
 * Host pipeline: compiler and executor above the backend. These mirror *
 * compiler::compile (src/compiler.rs:118-200) and exec::run_compiled   *
 * (src/exec.rs:334-452) for hosts that do not bring zeno's Rust front  *
 * half; the drop-in Rust path keeps its own and calls only the         *
 * backend entry points above.                                          *
 * ------------------------------------------------------------------ */

#define ZC_I_GATE 0
#define ZC_I_MEASURE 1
#define ZC_I_RESET 2
#define ZC_I_BARRIER 3

/* One program instruction (ir::Instr, src/ir.rs:36-52). cond_creg >= 0
 * wraps it in `if (creg == cond_value)` (Instr::If). */
typedef struct {
    int32_t kind;
    int32_t cond_creg;
    uint64_t cond_value;
    char name[8];
    uint32_t nq, np;
    uint32_t q[3];
    double p[3];
    uint32_t clbit;
    uint32_t _pad;
} zc_instr;

typedef struct {
    uint32_t fusion_max;  /* dense fusion width, 0..7 (0 disables all fusion) */
    uint32_t diag_max;    /* diagonal fusion width, <= 12 */
    uint32_t swap_perm;   /* 1: SWAP stays a zero-arithmetic permutation op */
} zc_compile_options;

#define ZC_OP_UNITARY 0
#define ZC_OP_DIAG 1
#define ZC_OP_CX 2
#define ZC_OP_MEASURE 3
#define ZC_OP_RESET 4
#define ZC_OP_SWAP 6

/* Read-only view of one compiled op (COp, src/compiler.rs:25-55). */
typedef struct {
    int32_t kind;
    uint32_t k;
    uint32_t qubits[12];
    const double *data; /* interleaved c64: 4^k (unitary) or 2^k (diagonal) entries */
    uint32_t a, b;      /* CX control/target, SWAP qubits, measure qubit/clbit */
    int32_t has_if;
    uint32_t creg_offset, creg_len;
    uint64_t value;
} zc_op_view;

typedef struct {
    uint32_t n_qubits, n_clbits;
    uint64_t nops, nfinal;
    int32_t dynamic;
    uint64_t input_gates, cancelled, output_ops, max_fused;
} zc_program_info;

typedef struct zc_program zc_program;

int zc_compile(uint32_t n_qubits, const uint32_t *creg_sizes, uint32_t n_cregs, const zc_instr *ins, size_t n_ins,
               const zc_compile_options *opt, zc_program **out);
void zc_program_free(zc_program *p);
int zc_program_get_info(const zc_program *p, zc_program_info *out);
int zc_program_get_op(const zc_program *p, size_t i, zc_op_view *out);
int zc_program_get_final(const zc_program *p, size_t i, uint32_t *qubit, uint32_t *clbit);

/* NoiseModel (src/noise.rs:39-47). */
typedef struct {
    double depolarizing_1q, depolarizing_2q, bit_flip, phase_flip, amplitude_damping, readout_flip_0to1,
        readout_flip_1to0;
} zc_noise;

typedef struct {
    int precision_bits;   /* 32, 64, or 0 = auto: f64 if it fits the budget, else f32 with zeno's
                             auto-precision notice (resolve_precision, src/exec.rs:261-304) */
    uint32_t flags;       /* ZC_FLAG_* for the backend */
    uint64_t shots;
    uint64_t seed;
    const zc_noise *noise; /* NULL or trivial: ideal simulation */
    double mem_fraction;   /* budget fraction of device memory (0.75 when 0) */
    uint32_t sweep_high;   /* sweep tile: high qubits per tile, 1..7 (0: automatic) */
    uint32_t _pad;
} zc_run_options;

typedef struct {
    int precision_bits;
    int batched;           /* 1: noisy shots ran in the batched trajectory engine */
    uint64_t n_keys;       /* distinct clbit words (keys[] filled up to cap) */
    double sim_seconds;    /* state allocation + gates + sampling (src/exec.rs:372-381) */
    uint64_t launches;
    uint64_t sweeps;
    uint64_t bytes_moved;
    char notices[512];     /* RunResult::notices (src/exec.rs:129), one per line, NUL-terminated */
} zc_run_result;

/* Run a compiled program. Counts are returned as (clbit word, count)
 * pairs sorted by clbit word; format keys with the program's cregs
 * (exec::format_key, src/exec.rs:235-253). `statevector` (2^n c64) may be
 * NULL; it is rejected for dynamic or noisy programs.
 *
 * Noisy or dynamic programs (mid-circuit measure, reset, conditioned ops)
 * at precision 32 run in the batched trajectory engine (no counterpart in
 * zeno, which replays shots one by one, src/exec.rs:459-619): every shot is
 * a trajectory with its own Philox4x32-10 stream (key = seed, counter =
 * (draw, shot)) and classical bits, all in one launch; the channel order of
 * src/noise.rs:145-175 and the measure/reset/condition semantics of
 * exec_shot_op are kept, results agree with zeno's per-shot path in
 * distribution. ZC_FLAG_PER_SHOT (or f64) selects the per-shot replay,
 * which reproduces zeno's RNG stream layout. */
int zc_run(const zc_program *p, const zc_run_options *opt, zc_run_result *res, uint64_t *keys, uint64_t *counts,
           size_t cap, double *statevector);

#ifdef __cplusplus
}
#endif
#endif
