// Batched trajectory engine: op encoding shared by host and kernel.
#pragma once
#include <stdint.h>

namespace zc {

enum : uint32_t { TOP_GATE = 0, TOP_MEASURE = 1, TOP_RESET = 2 };

// One op of a noisy or dynamic program. Gates: a dense 2^k x 2^k matrix
// (row-major, interleaved re/im f64, at mats + mat_off) on sorted qubits
// qs[0..k); CX and SWAP arrive as permutation matrices, diagonals as dense
// diagonals. Measure (qubit qs[0] into clbit) and reset (qubit qs[0]) carry
// k = 1 and the identity. `cond` makes the op run only if the classical
// bits [cond_off, cond_off + cond_len) equal cond_value (src/exec.rs:562-566).
struct TrajOp {
    uint32_t k;
    uint32_t qs[3];
    uint32_t mat_off;  // in doubles
    uint32_t kind;     // TOP_*
    uint32_t clbit;
    uint32_t cond;
    uint32_t cond_off, cond_len;
    uint64_t cond_value;
};

// NoiseModel fields in src/noise.rs order: dep1q, dep2q, bit flip,
// phase flip, amplitude damping, readout 0->1, readout 1->0.
struct TrajNoise {
    double p[7];
};

}  // namespace zc
