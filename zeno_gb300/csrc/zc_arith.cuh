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

// ------------------------------------------------------------------
// Double-float arithmetic for f64 states (fast mode).
//
// GB300 issues FP64 at 1/64 of the FP32 rate, so the f64 kernels' fast
// mode keeps the state in f64 in HBM but does the gate arithmetic on the
// FP32 pipe with unevaluated (hi, lo) float pairs (Dekker 1971; error-free
// TwoSum of Knuth, two-product via FMA). Conversions between f64 and the
// pair use integer and FP32 operations only, never the FP64 pipe. A general
// gate costs about 43 FP32 operations per output component and carries
// ~2^-46 relative error; f64 -> pair truncates at 2^-47, pair -> f64 rounds
// to nearest. Zero, subnormals and |x| < 2^-126 map to 0.

// f64 -> (hi, lo): hi = x truncated to 24 bits, lo = the next 23 bits.
__device__ __forceinline__ float2 df_from_f64(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const int e = (int)((hw >> 20) & 0x7ff);
    const unsigned sign = hw & 0x80000000u;
    const int ef = e - 896;   // f32 exponent field of hi
    const int efl = e - 919;  // exponent placing the low bits below hi
    const unsigned mant23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
    float hi = 0.0f, lo = 0.0f;
    if (ef >= 1 && ef <= 254) hi = __uint_as_float(sign | ((unsigned)ef << 23) | mant23);
    if (efl >= 1 && ef <= 254) {
        const unsigned top = sign | ((unsigned)efl << 23);
        lo = __fsub_rn(__uint_as_float(top | ((lw >> 6) & 0x7fffffu)), __uint_as_float(top));
    }
    return make_float2(hi, lo);
}

// Exact f32 -> f64 widening with integer operations only (the FP64 pipe's
// conversion shares its slow issue rate). Subnormals are normalised; inf and
// NaN keep their class.
__device__ __forceinline__ double f32_to_f64_exact(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned long long bits;
    if (e == 0xffu) {
        bits = sign | (0x7ffull << 52) | ((unsigned long long)m << 29);
    } else if (e != 0u) {
        bits = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    } else if (m == 0u) {
        bits = sign;
    } else {
        const int sh = __clz(m) - 8;  // brings the leading one to bit 23
        bits = sign | ((unsigned long long)(897 - sh) << 52) | ((unsigned long long)((m << sh) & 0x7fffffu) << 29);
    }
    return __longlong_as_double((long long)bits);
}
__device__ __forceinline__ double widen(double x) { return x; }
__device__ __forceinline__ double widen(float x) { return f32_to_f64_exact(x); }

// (hi, lo) -> f64 for |lo| <= ulp(hi): the f64 bit pattern of hi plus lo
// counted in f64 ulps of hi's binade (|lo| <= 2^28 of them; one binade lower
// when hi is a power of two and lo points down, where the ulp halves), scaled
// by a power of two and rounded to an integer: the f64 nearest hi + lo.
// |hi| < 2^-75 keeps hi alone; zero and subnormal hi give 0.
__device__ __forceinline__ double df_to_f64(float2 v) {
    const unsigned hb = __float_as_uint(v.x), lb = __float_as_uint(v.y);
    const unsigned eh = (hb >> 23) & 0xffu;
    if (eh == 0u) return 0.0;
    const unsigned mant = hb & 0x7fffffu;
    const unsigned long long hbits =
        ((unsigned long long)((hb & 0x80000000u) | ((eh + 896u) << 20) | (mant >> 3)) << 32) |
        (unsigned long long)(mant << 29);
    const bool down = mant == 0u && ((hb ^ lb) & 0x80000000u) && (lb & 0x7fffffffu);
    const unsigned se = 306u - eh + (down ? 1u : 0u);  // f32 exponent field of 2^(179 - eh (+1))
    if (se >= 255u) return __longlong_as_double((long long)hbits);
    const int L = __float2int_rn(__fmul_rn(v.y, __uint_as_float(se << 23)));
    return __longlong_as_double((long long)(hbits + (unsigned long long)(long long)((hb >> 31) ? -L : L)));
}

// Exact product split: a*b = p + e with e from one FMA, plus cross terms.
__device__ __forceinline__ void df_prod(float2 a, float2 b, float &p, float &e) {
    p = __fmul_rn(a.x, b.x);
    e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
}

// s + err = a + b exactly (TwoSum).
__device__ __forceinline__ float two_sum(float a, float b, float &err) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}

__device__ __forceinline__ float2 df_norm(float s, float lo) {
    const float h = __fadd_rn(s, lo);
    return make_float2(h, __fsub_rn(lo, __fsub_rn(h, s)));
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }

// x0*y0 + x1*y1 + x2*y2 + x3*y3 in double-float.
__device__ __forceinline__ float2 df_dot4(float2 x0, float2 y0, float2 x1, float2 y1, float2 x2, float2 y2, float2 x3,
                                          float2 y3) {
    float p0, e0, p1, e1, p2, e2, p3, e3, r1, r2, r3;
    df_prod(x0, y0, p0, e0);
    df_prod(x1, y1, p1, e1);
    df_prod(x2, y2, p2, e2);
    df_prod(x3, y3, p3, e3);
    float s = two_sum(p0, p1, r1);
    s = two_sum(s, p2, r2);
    s = two_sum(s, p3, r3);
    const float lo = __fadd_rn(__fadd_rn(__fadd_rn(r1, r2), r3), __fadd_rn(__fadd_rn(e0, e1), __fadd_rn(e2, e3)));
    return df_norm(s, lo);
}

__device__ __forceinline__ float2 df_dot2(float2 x0, float2 y0, float2 x1, float2 y1) {
    float p0, e0, p1, e1, r1;
    df_prod(x0, y0, p0, e0);
    df_prod(x1, y1, p1, e1);
    const float s = two_sum(p0, p1, r1);
    return df_norm(s, __fadd_rn(r1, __fadd_rn(e0, e1)));
}

// Gate matrix in double-float: m00r m00i m01r m01i m10r m10i m11r m11i.
struct MatDF {
    float2 v[8];
};

// Host-exact split of the f64 entries happens on the device once per op.
__device__ __forceinline__ MatDF df_matrix(const double *m) {
    MatDF r;
#pragma unroll
    for (int i = 0; i < 8; i++) r.v[i] = df_from_f64(m[i]);
    return r;
}

// 2x2 complex update of (a, b) in double-float (same formula as pair_update).
__device__ __forceinline__ void pair_update_df(const MatDF &m, float2 &ar, float2 &ai, float2 &br, float2 &bi) {
    const float2 nar = df_dot4(m.v[0], ar, df_neg(m.v[1]), ai, m.v[2], br, df_neg(m.v[3]), bi);
    const float2 nai = df_dot4(m.v[0], ai, m.v[1], ar, m.v[2], bi, m.v[3], br);
    const float2 nbr = df_dot4(m.v[4], ar, df_neg(m.v[5]), ai, m.v[6], br, df_neg(m.v[7]), bi);
    const float2 nbi = df_dot4(m.v[4], ai, m.v[5], ar, m.v[6], bi, m.v[7], br);
    ar = nar;
    ai = nai;
    br = nbr;
    bi = nbi;
}

// Real 2x2 update (r00 r01 r10 r11) of (a, b) in double-float: four
// two-term dot products instead of the complex update's four-term ones.
__device__ __forceinline__ void pair_update_rdf(const float2 *r, float2 &ar, float2 &ai, float2 &br, float2 &bi) {
    const float2 nar = df_dot2(r[0], ar, r[1], br);
    const float2 nai = df_dot2(r[0], ai, r[1], bi);
    const float2 nbr = df_dot2(r[2], ar, r[3], br);
    const float2 nbi = df_dot2(r[2], ai, r[3], bi);
    ar = nar;
    ai = nai;
    br = nbr;
    bi = nbi;
}

// x + t*y in double-float (one product, one TwoSum).
__device__ __forceinline__ float2 df_axpy(float2 x, float2 t, float2 y) {
    float p, e, r;
    df_prod(t, y, p, e);
    const float s = two_sum(x.x, p, r);
    return df_norm(s, __fadd_rn(x.y, __fadd_rn(e, r)));
}

// Unnormalised variants for chains of operations inside one register pass:
// the (s, lo) pair is left as TwoSum and the error terms give it (|lo| a few
// ulps of s at most); products and TwoSums of the next operation stay exact in
// their hi parts whatever the pair's normalisation, so the chain keeps the
// double-float error bound relative to its inputs. df_norm once at the end.
__device__ __forceinline__ float2 df_axpy_u(float2 x, float2 t, float2 y) {
    float p, e, r;
    df_prod(t, y, p, e);
    const float s = two_sum(x.x, p, r);
    return make_float2(s, __fadd_rn(x.y, __fadd_rn(e, r)));
}

__device__ __forceinline__ float2 df_dot2_u(float2 x0, float2 y0, float2 x1, float2 y1) {
    float p0, e0, p1, e1, r1;
    df_prod(x0, y0, p0, e0);
    df_prod(x1, y1, p1, e1);
    const float s = two_sum(p0, p1, r1);
    return make_float2(s, __fadd_rn(r1, __fadd_rn(e0, e1)));
}

__device__ __forceinline__ float2 df_renorm(float2 v) { return df_norm(v.x, v.y); }

__device__ __forceinline__ void cscale_df_u(float2 wr, float2 wi, float2 &ar, float2 &ai) {
    const float2 nr = df_dot2_u(wr, ar, df_neg(wi), ai);
    const float2 ni = df_dot2_u(wr, ai, wi, ar);
    ar = nr;
    ai = ni;
}

// Rotation update of (a, b) with unit diagonal: [[1, -t], [t, 1]]
// (|t| <= 1; the scale that makes it orthogonal lives in a diagonal).
__device__ __forceinline__ void pair_update_rot_df(float2 t, float2 &ar, float2 &ai, float2 &br, float2 &bi) {
    const float2 nt = df_neg(t);
    const float2 nar = df_axpy(ar, nt, br);
    const float2 nai = df_axpy(ai, nt, bi);
    const float2 nbr = df_axpy(br, t, ar);
    const float2 nbi = df_axpy(bi, t, ai);
    ar = nar;
    ai = nai;
    br = nbr;
    bi = nbi;
}

// The same rotation in T (FMA-contracted).
template <typename T>
__device__ __forceinline__ void pair_update_rot(T t, T &ar, T &ai, T &br, T &bi) {
    const T nar = rfma(-t, br, ar);
    const T nai = rfma(-t, bi, ai);
    const T nbr = rfma(t, ar, br);
    const T nbi = rfma(t, ai, bi);
    ar = nar;
    ai = nai;
    br = nbr;
    bi = nbi;
}

// The same real update in T (FMA-contracted).
template <typename T>
__device__ __forceinline__ void pair_update_real(const T *r, T &ar, T &ai, T &br, T &bi) {
    const T nar = rfma(r[0], ar, rmul(r[1], br));
    const T nai = rfma(r[0], ai, rmul(r[1], bi));
    const T nbr = rfma(r[2], ar, rmul(r[3], br));
    const T nbi = rfma(r[2], ai, rmul(r[3], bi));
    ar = nar;
    ai = nai;
    br = nbr;
    bi = nbi;
}

__device__ __forceinline__ void cscale_df(float2 wr, float2 wi, float2 &ar, float2 &ai) {
    const float2 nr = df_dot2(wr, ar, df_neg(wi), ai);
    const float2 ni = df_dot2(wr, ai, wi, ar);
    ar = nr;
    ai = ni;
}

// ------------------------------------------------------------------
// Packed double-float arithmetic (f32x2).
//
// add / sub / mul / fma .rn.f32x2 apply one IEEE FP32 operation to both
// halves of a 64-bit register pair. The FP32 datapath does the same number
// of operations per clock either way, but a packed instruction takes one
// issue slot and one step of a dependency chain for two of them. The
// double-float sweeps therefore hold a complex amplitude as
//   H = (re hi, im hi),  L = (re lo, im lo)
// and run the real and imaginary halves of a rotation through one
// instruction stream. Each half sees the operations of the scalar
// routines above in the same order; where a routine subtracts a product p,
// the packed one adds q = -p (negation is exact and rounding to nearest is
// symmetric), so both give the same values (a zero may carry the other
// sign).

__device__ __forceinline__ unsigned long long pk_bits(float2 v) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}
__device__ __forceinline__ float2 pk_float2(unsigned long long r) {
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk_bits(a)), "l"(pk_bits(b)));
    return pk_float2(d);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk_bits(a)), "l"(pk_bits(b)));
    return pk_float2(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk_bits(a)), "l"(pk_bits(b)));
    return pk_float2(d);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk_bits(a)), "l"(pk_bits(b)), "l"(pk_bits(c)));
    return pk_float2(d);
}

// A real double-float coefficient t as pairs: (t hi, t hi), (t lo, t lo),
// (-t hi, -t hi).
struct PkReal {
    float2 h, l, nh;
};

// [[1, -t], [t, 1]] on (a, b), unnormalised: per half, a - t b equals
// df_axpy_u(a, -t, b) and b + t a equals df_axpy_u(b, t, a). Both use the
// product of +t; q = -(t hi * y hi) serves the error term and the sums.
__device__ __forceinline__ void pk_rot_u(const PkReal &t, float2 &Ha, float2 &La, float2 &Hb, float2 &Lb) {
    // a - t b
    float2 q = mul2(t.nh, Hb);
    float2 e = fma2(t.h, Hb, q);
    e = fma2(t.h, Lb, e);
    e = fma2(t.l, Hb, e);  // t b = -q + e
    float2 s = add2(Ha, q);
    float2 bb = sub2(s, Ha);
    float2 r = add2(sub2(Ha, sub2(s, bb)), sub2(q, bb));
    const float2 nHa = s, nLa = add2(La, sub2(r, e));
    // b + t a
    q = mul2(t.nh, Ha);
    e = fma2(t.h, Ha, q);
    e = fma2(t.h, La, e);
    e = fma2(t.l, Ha, e);  // t a = -q + e
    s = sub2(Hb, q);
    bb = sub2(s, Hb);
    r = sub2(sub2(Hb, sub2(s, bb)), add2(q, bb));
    Lb = add2(Lb, add2(e, r));
    Hb = s;
    Ha = nHa;
    La = nLa;
}

// (H, L) <-> the scalar routines' (re, im) double-float pairs.
__device__ __forceinline__ void pk_split(float2 H, float2 L, float2 &ar, float2 &ai) {
    ar = make_float2(H.x, L.x);
    ai = make_float2(H.y, L.y);
}
__device__ __forceinline__ void pk_join(float2 ar, float2 ai, float2 &H, float2 &L) {
    H = make_float2(ar.x, ai.x);
    L = make_float2(ar.y, ai.y);
}

// Renormalise both halves (df_norm per half).
__device__ __forceinline__ void pk_renorm(float2 &H, float2 &L) {
    const float2 h = add2(H, L);
    L = sub2(L, sub2(h, H));
    H = h;
}

// f64 (re, im) <-> packed pairs; to_f64 renormalises first.
__device__ __forceinline__ void pk_from_f64(double re, double im, float2 &H, float2 &L) {
    pk_join(df_from_f64(re), df_from_f64(im), H, L);
}
__device__ __forceinline__ void pk_to_f64(float2 H, float2 L, double &re, double &im) {
    pk_renorm(H, L);
    re = df_to_f64(make_float2(H.x, L.x));
    im = df_to_f64(make_float2(H.y, L.y));
}

// Arithmetic policies: 0 = exact reference trees, 1 = FMA-contracted,
// 2 = double-float on the FP32 pipe (f64 states only).
enum : int { AR_EXACT = 0, AR_FMA = 1, AR_DF = 2 };

// pair_update under policy A on values stored as T.
template <typename T, int A>
__device__ __forceinline__ void upd2(const Mat2<T> &m, const MatDF &md, T &ar, T &ai, T &br, T &bi) {
    if constexpr (A == AR_DF) {
        float2 xr = df_from_f64(ar), xi = df_from_f64(ai), yr = df_from_f64(br), yi = df_from_f64(bi);
        pair_update_df(md, xr, xi, yr, yi);
        ar = df_to_f64(xr);
        ai = df_to_f64(xi);
        br = df_to_f64(yr);
        bi = df_to_f64(yi);
    } else {
        pair_update<T, A == AR_EXACT>(m, ar, ai, br, bi);
    }
}

template <typename T, int A>
__device__ __forceinline__ void scale2(T wr, T wi, float2 wrd, float2 wid, T &ar, T &ai) {
    if constexpr (A == AR_DF) {
        float2 xr = df_from_f64(ar), xi = df_from_f64(ai);
        cscale_df(wrd, wid, xr, xi);
        ar = df_to_f64(xr);
        ai = df_to_f64(xi);
    } else {
        cscale<T, A == AR_EXACT>(wr, wi, ar, ai);
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
