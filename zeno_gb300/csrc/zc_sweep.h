// Shared definitions of the multi-op sweep kernel and its host scheduler.
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace zc {

constexpr uint32_t kOuterFlag = 0x80000000u;  // operand names a non-local qubit (global position)
constexpr int kMaxMicroOps = 40;               // ops per sweep
constexpr uint32_t kMaxSweepHigh = 7;          // chosen high qubits per tile
constexpr size_t kSweepSmemBytes = 64 * 1024;  // one tile buffer: 2^12 f64 or 2^13 f32 (re + im)

enum : uint32_t { MOP_U1 = 1, MOP_D1 = 2, MOP_DK = 3, MOP_CX = 4, MOP_SWAP = 5, MOP_R1 = 6, MOP_RT = 7 };

// Tile geometry: local qubits are 0..L-1 plus hpos[0..H) (ascending).
// form (double-float sweeps of f64 states): kFormInDf — the state holds
// packed float pairs on entry (the previous sweep left them: re slot
// (re hi, im hi), im slot (re lo, im lo)); kFormOutDf — leave normalised
// pairs for the next sweep instead of rounding to f64.
constexpr uint32_t kFormInDf = 1u, kFormOutDf = 2u;
struct SweepGeom {
    uint32_t n, L, H, form;
    uint32_t hpos[16];
    uint64_t ntiles;
};

// One op inside a sweep, operands as local bit indices (0..L+H) or
// kOuterFlag | global qubit. U1: a = bit, m = 2x2 row-major (re, im);
// D1: a = bit, m[0..4) = d0, d1; DK: k, loc[], table = byte offset of 2^k
// (re, im) pairs in the sweep's table block (for double-float sweeps of f64
// states: 2^k entries of (re hi, re lo, im hi, im lo) floats);
// CX: a = control, b = target (local); SWAP: a, b local; R1: a = bit,
// m[0..4) = real 2x2 r00 r01 r10 r11; RT: a = bit, m[0] = t, b = flip:
// [[1, -t], [t, 1]], then (flip) the pair's two amplitudes trade places.
struct MicroOp {
    uint32_t kind, a, b, k;
    uint32_t loc[12];
    uint64_t table;
    double m[8];
};

// Packed launch over many states: header, then jobs, then each job's
// micro-ops and tables at the given byte offsets of the same blob.
struct SweepBatch {
    uint32_t njobs, pad;
    uint64_t total_tiles;
};

struct SweepJob {
    void *re, *im;  // the state's device arrays
    uint32_t L, H, nops, pad;
    uint32_t hpos[8];
    uint64_t ntiles;
    uint64_t tile_start;  // first tile of this job in the packed index space
    uint64_t ops_off;     // byte offset of its MicroOps in the blob (16-byte aligned)
    uint64_t tables_off;  // byte offset of its tables in the blob
};

}  // namespace zc
