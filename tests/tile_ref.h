// Sequential reference for the host checks of the sweep kernel's tile logic
// (passes_harness.cpp): micro-ops applied one at a time
// to one tile of 2^g_tile_bits amplitudes in complex<double>, and a generator
// of random micro-op lists shaped like the planner's.
#pragma once
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "zc_passes.h"

namespace tile_ref {

using cd = std::complex<double>;
using zc::OpHead;

inline uint32_t g_tile_bits = 9;  // set_tile_bits() changes both
inline uint32_t g_size = 1u << 9;
inline void set_tile_bits(uint32_t bits) {
    g_tile_bits = bits;
    g_size = 1u << bits;
}
constexpr uint32_t kOuter0 = 20, kNOuter = 6;  // outer qubits 20..25
inline uint64_t g_base = 0;                    // the tile's outer qubit values

struct Op {
    OpHead h;
    double m[8];
    std::vector<cd> tab;  // DK table
};

inline uint32_t bit_of(uint32_t slot, uint32_t x) {
    return x & zc::kOuterFlag ? (uint32_t)((g_base >> (x & ~zc::kOuterFlag)) & 1) : (slot >> x) & 1;
}

inline void apply_pair(std::vector<cd> &s, uint32_t a, const cd u[4]) {
    for (uint32_t i = 0; i < g_size; i++)
        if (!((i >> a) & 1)) {
            const uint32_t j = i | (1u << a);
            const cd x = s[i], y = s[j];
            s[i] = u[0] * x + u[1] * y;
            s[j] = u[2] * x + u[3] * y;
        }
}

// The 2x2 matrix of a one-qubit op; RT rows swapped when flipped.
inline void gate_matrix(const Op &op, cd u[4]) {
    const OpHead &h = op.h;
    if (h.kind == zc::MOP_U1) {
        for (int i = 0; i < 4; i++) u[i] = cd(op.m[2 * i], op.m[2 * i + 1]);
    } else if (h.kind == zc::MOP_R1) {
        for (int i = 0; i < 4; i++) u[i] = op.m[i];
    } else {  // RT: [[1, -t], [t, 1]]
        const double t = op.m[0];
        const cd r[4] = {1.0, -t, t, 1.0};
        if (h.b) {
            u[0] = r[2], u[1] = r[3], u[2] = r[0], u[3] = r[1];
        } else {
            for (int i = 0; i < 4; i++) u[i] = r[i];
        }
    }
}

// Table entry of a diagonal op (D1: m = d0r d0i d1r d1i; DK: tab).
inline cd diag_entry(const Op &op, uint32_t u) {
    if (op.h.kind == zc::MOP_D1) {
        const uint32_t one = bit_of(u, op.h.a);
        return cd(op.m[2 * one], op.m[2 * one + 1]);
    }
    uint32_t j = 0;
    for (uint32_t b = 0; b < op.h.k; b++) j |= bit_of(u, op.h.loc[b]) << b;
    return op.tab[j];
}

inline void apply_one(std::vector<cd> &s, const Op &op) {
    const OpHead &h = op.h;
    switch (h.kind) {
        case zc::MOP_U1:
        case zc::MOP_R1:
        case zc::MOP_RT: {
            cd u[4];
            gate_matrix(op, u);
            apply_pair(s, h.a, u);
            break;
        }
        case zc::MOP_D1:
        case zc::MOP_DK:
            for (uint32_t i = 0; i < g_size; i++) s[i] *= diag_entry(op, i);
            break;
        case zc::MOP_CX:
            for (uint32_t i = 0; i < g_size; i++)
                if (bit_of(i, h.a) && !((i >> h.b) & 1)) std::swap(s[i], s[i | (1u << h.b)]);
            break;
        case zc::MOP_SWAP:
            for (uint32_t i = 0; i < g_size; i++)
                if (((i >> h.a) & 1) && !((i >> h.b) & 1)) std::swap(s[i], s[(i ^ (1u << h.a)) | (1u << h.b)]);
            break;
    }
}

// Random micro-op list: one-qubit gates (rotations, real and complex 2x2),
// table diagonals with local and outer support, CX with local or outer
// controls, SWAP; often a CX block, a diagonal and a
// run of gates on the CX targets, the shape the double-float lowering emits.
struct Gen {
    std::mt19937_64 rng;
    std::uniform_real_distribution<double> U{-1.0, 1.0};
    uint32_t tables = 0;
    explicit Gen(uint64_t seed) : rng(seed) {}
    uint32_t local() { return (uint32_t)(rng() % g_tile_bits); }
    uint32_t outer() { return zc::kOuterFlag | (kOuter0 + (uint32_t)(rng() % kNOuter)); }
    void new_base() {
        g_base = 0;
        for (uint32_t i = 0; i < kNOuter; i++)
            if (rng() & 1) g_base |= 1ull << (kOuter0 + i);
    }
    void gate(std::vector<Op> &ops, uint32_t a) {
        Op op{};
        const int kind = (int)(rng() % 6);
        op.h.a = a;
        if (kind < 4) {
            op.h.kind = zc::MOP_RT;
            op.m[0] = U(rng);
            op.h.b = (uint32_t)(rng() & 1);
        } else if (kind < 5) {
            op.h.kind = zc::MOP_R1;
            for (int i = 0; i < 4; i++) op.m[i] = U(rng);
        } else {
            op.h.kind = zc::MOP_U1;
            for (int i = 0; i < 8; i++) op.m[i] = U(rng);
        }
        ops.push_back(op);
    }
    void dk(std::vector<Op> &ops) {
        Op op{};
        op.h.kind = zc::MOP_DK;
        op.h.k = 1 + (uint32_t)(rng() % 6);
        uint64_t used = 0;
        for (uint32_t b = 0; b < op.h.k;) {
            const uint32_t x = rng() % 4 == 0 ? outer() : local();
            const uint64_t key = x & zc::kOuterFlag ? 1ull << (32 + (x & 31)) : 1ull << x;
            if (used & key) continue;
            used |= key;
            op.h.loc[b++] = x;
        }
        op.h.table = tables++;
        op.tab.resize((size_t)1 << op.h.k);
        for (auto &w : op.tab) w = std::polar(1.0, 3.0 * U(rng));
        ops.push_back(op);
    }
    void cx(std::vector<Op> &ops, uint32_t t) {
        Op op{};
        op.h.kind = zc::MOP_CX;
        op.h.b = t;
        do op.h.a = rng() % 3 == 0 ? outer() : local();
        while (op.h.a == t);
        ops.push_back(op);
    }
    void swap(std::vector<Op> &ops) {
        Op op{};
        op.h.kind = zc::MOP_SWAP;
        op.h.a = local();
        do op.h.b = local();
        while (op.h.b == op.h.a);
        ops.push_back(op);
    }
    std::vector<Op> list(int max_len) {
        std::vector<Op> ops;
        tables = 0;
        const int len = 4 + (int)(rng() % (uint64_t)max_len);
        while ((int)ops.size() < len) {
            const int r = (int)(rng() % 10);
            if (r < 4) {
                uint32_t t[3];
                const int g = 1 + (int)(rng() % 3);
                for (int i = 0; i < g; i++) {
                    bool fresh;
                    do {
                        t[i] = local();
                        fresh = true;
                        for (int j = 0; j < i; j++) fresh &= t[j] != t[i];
                    } while (!fresh);
                }
                const int ncx = (int)(rng() % 4);
                for (int i = 0; i < ncx; i++) cx(ops, t[rng() % g]);
                if (rng() % 3) dk(ops);
                for (int i = 0; i < g; i++) gate(ops, t[i]);
            } else if (r < 6) {
                gate(ops, local());
            } else if (r < 7) {
                dk(ops);
            } else if (r < 9) {
                cx(ops, local());
            } else {
                swap(ops);
            }
        }
        return ops;
    }
};

inline double rel_diff(const std::vector<cd> &got, const std::vector<cd> &want) {
    double err = 0.0, scale = 0.0;
    for (size_t i = 0; i < want.size(); i++) {
        err = std::max(err, std::abs(got[i] - want[i]));
        scale = std::max(scale, std::abs(want[i]));
    }
    return err / scale;
}

}  // namespace tile_ref
