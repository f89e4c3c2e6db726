/*
 * zeno_oracle.h — CPU oracle for the zeno state-vector hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * simulator's scalar CPU backend, sampler, executor, noise channels, gate
 * library and fusion compiler. It exists to check the CUDA backend and to
 * time the CPU baseline. Nothing in the shipped library links or calls it.
 *
 * Reference files restated (paths inside the zeno project):
 *   src/state.rs    scalar kernels (kern_1q_scalar :232-260, kern_kq_scalar
 *                   :355-392, apply_cx :397-417, kern_diag1_scalar :498-527,
 *                   kern_diagk_scalar :577-596, prob_one :599-626,
 *                   collapse :630-661, norm_sqr :143-156)
 *   src/sample.rs   sample_indices :29-111
 *   src/exec.rs     CpuBackend :164-225, splitmix64 :227-232, run_sampled
 *                   :407-452, run_per_shot :459-549, exec_shot_op :556-619
 *   src/noise.rs    apply_pauli :91-100, amplitude_damp :114-127,
 *                   apply_gate_noise :145-175, readout_flip :181-192
 *   src/gates.rs    lookup :101-115, build :119-188
 *   src/compiler.rs compile :118-200, cancel :215-239, lower_gate :296-347,
 *                   permute_*_to_sorted :370-398, embed_* / matmul :421-471,
 *                   fuse_diagonals :477-535, fuse_general :540-626
 *   src/mem.rs      state_bytes / max_qubits / plan :79-131
 *
 * Third-party arithmetic restated from published definitions: xoshiro256++
 * and splitmix64 (Blackman & Vigna), rand_xoshiro 0.6 seed_from_u64
 * (SplitMix64 fill), rand 0.8.5 Standard f64 (53-bit) and
 * UniformInt<u64>::sample_single (widening-multiply rejection).
 *
 * Parity pinning: the reference ships no golden amplitude or count vectors,
 * so this oracle is pinned by the reference's known-answer tests (QFT vs
 * DFT formula, GHZ two-branch, examples/qft.qasm round trip, gate-library
 * identities, 6-sigma statistics, noise closed forms) and by an independent
 * dense simulator (zo_refsim_*). Bit-exact RNG/count parity with the Rust
 * binary itself is unpinned: the Rust toolchain and crates are absent.
 */
#ifndef ZENO_ORACLE_H
#define ZENO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double re, im;
} zo_c64;

/* ---------------------------------------------------------------- RNG */
typedef struct {
    uint64_t s[4];
} zo_rng;

uint64_t zo_splitmix64(uint64_t x);
void zo_rng_seed(zo_rng *r, uint64_t seed);
uint64_t zo_rng_next(zo_rng *r);
double zo_rng_f64(zo_rng *r);
uint64_t zo_rng_range(zo_rng *r, uint64_t lo, uint64_t hi); /* [lo, hi) */

/* -------------------------------------------------------------- gates */
/* kind: 0 unitary (dim*dim entries), 1 diagonal (dim entries).
 * Returns arity (>0) or 0 for an unknown name / wrong parameter count. */
int zo_gate_build(const char *name, const double *params, int np, int *kind, zo_c64 *out);
int zo_gate_lookup(const char *name, int *arity, int *nparams);

/* ----------------------------------------------------------- program */
enum { ZO_I_GATE = 0, ZO_I_MEASURE = 1, ZO_I_RESET = 2, ZO_I_BARRIER = 3 };

typedef struct {
    int32_t kind;      /* ZO_I_* */
    int32_t cond_creg; /* -1: unconditional; else `if (creg == cond_value)` */
    uint64_t cond_value;
    char name[8];
    uint32_t nq, np;
    uint32_t q[3];
    double p[3];
    uint32_t clbit;
    uint32_t _pad;
} zo_instr;

/* ------------------------------------------------------ compiled ops */
enum { ZO_OP_UNITARY = 0, ZO_OP_DIAG = 1, ZO_OP_CX = 2, ZO_OP_MEASURE = 3, ZO_OP_RESET = 4, ZO_OP_BARRIER = 5 };

#define ZO_MAXQ 12

typedef struct {
    int32_t kind;
    uint32_t k;                /* support size for unitary / diagonal */
    uint32_t qubits[ZO_MAXQ];  /* sorted support */
    zo_c64 *data;              /* owned: dim*dim (unitary) or dim (diag) */
    uint32_t control, target;  /* CX */
    uint32_t qubit, clbit;     /* measure / reset */
    int32_t has_if;            /* COp::If wrapper around this op */
    uint32_t creg_offset, creg_len;
    uint64_t value;
} zo_op;

typedef struct {
    uint64_t input_gates, cancelled, output_ops, max_fused;
} zo_stats;

typedef struct zo_compiled zo_compiled;

/* Returns 0 on success; on error returns nonzero and writes a message. */
int zo_compile(uint32_t n_qubits, const uint32_t *creg_sizes, uint32_t n_cregs, const zo_instr *ins,
               size_t n_ins, uint32_t fusion_max, uint32_t diag_max, zo_compiled **out, char *err,
               size_t err_len);
void zo_compiled_free(zo_compiled *c);
size_t zo_compiled_nops(const zo_compiled *c);
const zo_op *zo_compiled_op(const zo_compiled *c, size_t i);
int zo_compiled_dynamic(const zo_compiled *c);
size_t zo_compiled_nfinal(const zo_compiled *c);
void zo_compiled_final(const zo_compiled *c, size_t i, uint32_t *qubit, uint32_t *clbit);
void zo_compiled_stats(const zo_compiled *c, zo_stats *s);

/* ------------------------------------------------------ CPU backend */
typedef struct zo_state zo_state;

zo_state *zo_state_new(uint32_t n_qubits, int prec_bits);
void zo_state_free(zo_state *s);
void zo_set_threads(int threads);
int zo_get_threads(void);
void zo_apply_unitary(zo_state *s, const uint32_t *qs, uint32_t k, const zo_c64 *mat);
void zo_apply_diagonal(zo_state *s, const uint32_t *qs, uint32_t k, const zo_c64 *d);
void zo_apply_cx(zo_state *s, uint32_t control, uint32_t target);
double zo_prob_one(zo_state *s, uint32_t q);
int zo_measure(zo_state *s, uint32_t q, double u);
void zo_reset_all(zo_state *s);
void zo_sample(zo_state *s, uint64_t shots, uint64_t seed, uint64_t *out);
void zo_statevector(zo_state *s, zo_c64 *out);
double zo_norm_sqr(zo_state *s);
/* Raw access for tests: load an arbitrary state (interleaved c64). */
void zo_load_state(zo_state *s, const zo_c64 *in);

/* -------------------------------------------------------- executor */
typedef struct {
    double depolarizing_1q, depolarizing_2q, bit_flip, phase_flip, amplitude_damping,
        readout_flip_0to1, readout_flip_1to0;
} zo_noise;

/* Run a compiled circuit (exec.rs run_inner minus precision resolution).
 * Writes up to cap (clbit word, count) pairs sorted by clbit word and
 * returns the number of distinct keys, or -1 on error. A non-null noise
 * model that is non-trivial selects the per-shot trajectory path. */
long zo_run(const zo_compiled *c, int prec_bits, uint64_t shots, uint64_t seed, const zo_noise *noise,
            uint64_t *keys, uint64_t *counts, size_t cap, zo_c64 *statevector_out);

/* --------------------------------------------------------- mem.rs */
uint64_t zo_state_bytes(uint32_t n, int prec_bits);
uint32_t zo_max_qubits(uint64_t budget, int prec_bits);

/* -------------------------------------- independent dense simulator */
/* Interleaved amplitudes, textbook gather/matvec/scatter with complex
 * arithmetic (a second, structurally different oracle). Qubits are in
 * argument order: bit b of the local index is qs[b]. */
void zo_refsim_apply(zo_c64 *amps, uint32_t n, const uint32_t *qs, uint32_t k, const zo_c64 *mat);

#ifdef __cplusplus
}
#endif
#endif
