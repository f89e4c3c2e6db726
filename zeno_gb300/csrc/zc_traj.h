// Batched trajectory engine: op encoding shared by host and kernel.
#pragma once
#include <stdint.h>

namespace zc {

// One gate of a noisy program: a dense 2^k x 2^k matrix (row-major,
// interleaved re/im f64, at mats + mat_off) on sorted qubits qs[0..k).
// CX and SWAP arrive as permutation matrices, diagonals as dense diagonals.
struct TrajOp {
    uint32_t k;
    uint32_t qs[3];
    uint32_t mat_off;  // in doubles
};

// NoiseModel fields in src/noise.rs order: dep1q, dep2q, bit flip,
// phase flip, amplitude damping, readout 0->1, readout 1->0.
struct TrajNoise {
    double p[7];
};

}  // namespace zc
