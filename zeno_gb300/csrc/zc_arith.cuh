// Arithmetic policy for the gate kernels.
//
// EXACT = true reproduces zeno's scalar CPU kernels bit for bit: every
// product and sum is a separately rounded IEEE operation (the __*_rn
// intrinsics are never contracted into FMA), evaluated in the reference's
// left-to-right order (src/state.rs:253-256, :382-383, :521-525, :592-593).
// EXACT = false lets the update use fused multiply-adds (tolerance parity).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace zc {

template <typename T>
struct Vec;
template <>
struct Vec<double> {
    using type = double2;  // 16-byte vector access
    static constexpr int N = 2;
};
template <>
struct Vec<float> {
    using type = float4;
    static constexpr int N = 4;
};

__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <typename T>
struct Mat2 {
    T v[8];  // m00r m00i m01r m01i m10r m10i m11r m11i
};

// 2x2 complex update of the pair (a, b) = (bit q clear, bit q set)
// (kern_1q_scalar, src/state.rs:251-257).
template <typename T, bool EXACT>
__device__ __forceinline__ void pair_update(const Mat2<T> &m, T &ar, T &ai, T &br, T &bi) {
    const T m00r = m.v[0], m00i = m.v[1], m01r = m.v[2], m01i = m.v[3];
    const T m10r = m.v[4], m10i = m.v[5], m11r = m.v[6], m11i = m.v[7];
    T nar, nai, nbr, nbi;
    if constexpr (EXACT) {
        nar = rsub(radd(rsub(rmul(m00r, ar), rmul(m00i, ai)), rmul(m01r, br)), rmul(m01i, bi));
        nai = radd(radd(radd(rmul(m00r, ai), rmul(m00i, ar)), rmul(m01r, bi)), rmul(m01i, br));
        nbr = rsub(radd(rsub(rmul(m10r, ar), rmul(m10i, ai)), rmul(m11r, br)), rmul(m11i, bi));
        nbi = radd(radd(radd(rmul(m10r, ai), rmul(m10i, ar)), rmul(m11r, bi)), rmul(m11i, br));
    } else {
        nar = rfma(-m01i, bi, rfma(m01r, br, rfma(-m00i, ai, m00r * ar)));
        nai = rfma(m01i, br, rfma(m01r, bi, rfma(m00i, ar, m00r * ai)));
        nbr = rfma(-m11i, bi, rfma(m11r, br, rfma(-m10i, ai, m10r * ar)));
        nbi = rfma(m11i, br, rfma(m11r, bi, rfma(m10i, ar, m10r * ai)));
    }
    ar = nar;
    ai = nai;
    br = nbr;
    bi = nbi;
}

// Complex scale of one amplitude by (wr, wi) (kern_diag*_scalar,
// src/state.rs:521-525, :592-593): re' = wr*ar - wi*ai, im' = wr*ai + wi*ar.
template <typename T, bool EXACT>
__device__ __forceinline__ void cscale(T wr, T wi, T &ar, T &ai) {
    T nr, ni;
    if constexpr (EXACT) {
        nr = rsub(rmul(wr, ar), rmul(wi, ai));
        ni = radd(rmul(wr, ai), rmul(wi, ar));
    } else {
        nr = rfma(-wi, ai, wr * ar);
        ni = rfma(wi, ar, wr * ai);
    }
    ar = nr;
    ai = ni;
}

// One term of the fused k-qubit matvec (kern_kq_scalar, src/state.rs:382-383):
// ar = (ar + wr*xr) - wi*xi ; ai = (ai + wr*xi) + wi*xr.
template <typename T, bool EXACT>
__device__ __forceinline__ void cmac(T wr, T wi, T xr, T xi, T &ar, T &ai) {
    if constexpr (EXACT) {
        ar = rsub(radd(ar, rmul(wr, xr)), rmul(wi, xi));
        ai = radd(radd(ai, rmul(wr, xi)), rmul(wi, xr));
    } else {
        ar = rfma(-wi, xi, rfma(wr, xr, ar));
        ai = rfma(wi, xr, rfma(wr, xi, ai));
    }
}

// insert_zeros (src/state.rs:162-169): spread g around zero bits at the
// ascending positions qs[0..k).
__device__ __forceinline__ uint64_t insert_zeros(uint64_t g, const uint32_t *qs, int k) {
    uint64_t x = g;
    for (int i = 0; i < k; i++) {
        const uint32_t q = qs[i];
        const uint64_t low = x & ((1ull << q) - 1);
        x = ((x >> q) << (q + 1)) | low;
    }
    return x;
}

__device__ __forceinline__ uint64_t insert_zero(uint64_t h, uint32_t q) {
    return ((h >> q) << (q + 1)) | (h & ((1ull << q) - 1));
}

}  // namespace zc
