/*
 * zeno_cuda_serve.h — continuous-batching serving engine over the GB300
 * state-vector backend (no counterpart in zeno, which runs one circuit per
 * call: src/lib.rs:248, src/exec.rs:407-452).
 *
 * A server owns one HBM pool. Requests (compiled static programs) are
 * admitted FIFO as their state fits the pool and a slot is free; every step
 * advances all admitted requests together in one packed launch (a captured
 * CUDA graph replayed with the step's job list), samples the requests that
 * finished with the same sampler and seed semantics as zc_sample /
 * zc_run, and frees their slots. Results are sampled basis indices
 * (ascending), mapped to clbits by the program's final measurements.
 */
#ifndef ZENO_CUDA_SERVE_H
#define ZENO_CUDA_SERVE_H

#include "zeno_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    uint64_t pool_bytes; /* device pool for request states (0: half the device budget) */
    uint32_t max_slots;  /* requests resident at once (0: 1024) */
    uint32_t flags;      /* ZC_FLAG_EXACT or ZC_FLAG_FAST */
} zc_server_options;

typedef struct {
    uint64_t pending, active, done;
    uint64_t launches, packed_launches, admitted, completed;
    uint64_t pool_used;
    uint64_t steps;
    /* cumulative host microseconds: planning + launching the packed steps,
     * sampling finished requests, waiting for the device at step ends */
    uint64_t plan_us, sample_us, wait_us;
    /* cumulative device microseconds between each step's first and last
     * launch (CUDA events on the server stream) */
    uint64_t device_us;
} zc_server_status;

typedef struct zc_server zc_server;

int zc_server_create(const zc_server_options *opt, zc_server **out);
void zc_server_destroy(zc_server *s);
/* Queue a request; its program must be static (no mid-circuit measure,
 * reset or if). precision_bits 32 or 64 (f64 escalation); <= 30 qubits,
 * <= 65536 shots. The program may be freed after this returns. */
int zc_server_submit(zc_server *s, const zc_program *p, int precision_bits, uint64_t shots, uint64_t seed,
                     uint64_t *request_id);
/* Admit, run one packed step, complete finished requests; synchronises. */
int zc_server_step(zc_server *s, zc_server_status *status);
/* Ids of finished requests not yet taken. */
int zc_server_done_ids(zc_server *s, uint64_t *ids, size_t cap, size_t *n);
/* Copy a finished request's sampled indices (up to cap) and release it. */
int zc_server_take(zc_server *s, uint64_t request_id, uint64_t *indices, uint64_t cap, uint64_t *n);

#ifdef __cplusplus
}
#endif
#endif
