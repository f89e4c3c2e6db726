// Batched noisy trajectories: every trajectory of a noisy run in ONE launch.
//
// zeno runs a noisy circuit one shot at a time (src/exec.rs:459-549): each
// shot replays the ops and, after every gate, the channels of
// src/noise.rs:145-175 — depolarizing, then per touched qubit bit flip,
// phase flip and amplitude damping (whose jump probability gamma * P(1)
// needs a reduction over the state), then readout flips at measurement.
//
// Here a persistent CTA owns one trajectory at a time; its state (2^n
// amplitudes) stays in a per-CTA buffer that fits in L2. Per op the CTA
// makes one pass over the state that (a) applies the previous op's pending
// noise operators that are diagonal as a per-element factor, (b) applies the
// gate (times the depolarizing Pauli string drawn for this op), and
// (c) accumulates the joint probability table of the op's qubits. Thread 0
// then resolves flips and damping for the touched qubits in the reference's
// order on that table (each decision updates the table) and leaves the
// resulting 2x2 operators pending for the next pass. All draws of an op are
// independent of the state, so they are taken up front in the reference's
// order from a per-trajectory Philox4x32-10 stream (zc_philox.h).
// Probabilities are summed in double-float per thread and reduced in FP64.
#include <algorithm>

#include "zc_arith.cuh"
#include "zc_internal.h"
#include "zc_philox.h"
#include "zc_traj.h"

namespace zc {
namespace {

constexpr int kTrajThreads = 256;  // four CTAs (trajectories) per SM at 64 registers

// ---------------------------------------------------------------- complex helpers

// Complex values of the per-op operators (gate x Pauli string, pending noise
// operators, diagonal factors): single precision, like the f32 states they act
// on (GB300's FP64 pipe would make thread 0's serial work the bottleneck);
// branch probabilities stay FP64.
struct C2 {
    float re, im;
};
__device__ __forceinline__ C2 cmul(C2 a, C2 b) { return C2{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return C2{a.re + b.re, a.im + b.im}; }

// Pauli by code 1 = X, 2 = Y, 3 = Z as a 2x2 row-major complex matrix.
__device__ void pauli(int code, C2 *m) {
    for (int i = 0; i < 4; i++) m[i] = C2{0, 0};
    if (code == 1) m[1] = m[2] = C2{1, 0};
    if (code == 2) m[1] = C2{0, -1}, m[2] = C2{0, 1};
    if (code == 3) m[0] = C2{1, 0}, m[3] = C2{-1, 0};
    if (code == 0) m[0] = m[3] = C2{1, 0};
}

// out = a . b for 2x2.
__device__ void mul22(const C2 *a, const C2 *b, C2 *out) {
    C2 r[4];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) r[i * 2 + j] = cadd(cmul(a[i * 2], b[j]), cmul(a[i * 2 + 1], b[2 + j]));
    for (int i = 0; i < 4; i++) out[i] = r[i];
}

struct Pending {
    uint32_t q;
    C2 m[4];
};

struct Shared {
    float mr[64], mi[64];        // current op matrix (gate x Pauli string), f32
    double J[8];                  // joint probability table of the op's qubits
    Pending pend[3];              // operators left by the previous op's noise
    int npend;
    uint32_t dq[3];               // qubits of diagonal pending factors
    float dr[8], di[8];           // per-element factor table over dq bits
    int nd;
    int nondiag;                  // some pending operator is not diagonal
    double red[kTrajThreads / 32][8];
    double seg[kTrajThreads];
    uint64_t draw;                // next draw number of this trajectory
    uint64_t pick;                // sampled basis index
    uint64_t cl;                  // classical bits of this trajectory
    int skip;                     // the current op's condition is false
    int fail;
};

// Apply every non-diagonal pending operator as a 1-qubit pass.
template <typename T>
__device__ void apply_nondiag_pending(T *re, T *im, uint32_t n, Shared &s) {
    const uint64_t half = 1ull << (n - 1);
    for (int p = 0; p < s.npend; p++) {
        const Pending &P = s.pend[p];
        if (P.m[1].re == 0 && P.m[1].im == 0 && P.m[2].re == 0 && P.m[2].im == 0) continue;
        const float m00r = P.m[0].re, m00i = P.m[0].im, m01r = P.m[1].re, m01i = P.m[1].im;
        const float m10r = P.m[2].re, m10i = P.m[2].im, m11r = P.m[3].re, m11i = P.m[3].im;
        for (uint64_t h = threadIdx.x; h < half; h += blockDim.x) {
            const uint64_t a = insert_zero(h, P.q), b = a | (1ull << P.q);
            const float ar = re[a], ai = im[a], br = re[b], bi = im[b];
            re[a] = m00r * ar - m00i * ai + m01r * br - m01i * bi;
            im[a] = m00r * ai + m00i * ar + m01r * bi + m01i * br;
            re[b] = m10r * ar - m10i * ai + m11r * br - m11i * bi;
            im[b] = m10r * ai + m10i * ar + m11r * bi + m11i * br;
        }
        __syncthreads();
    }
}

// Per-element factor of the diagonal pending operators.
__device__ __forceinline__ void diag_factor(const Shared &s, uint64_t idx, float &fr, float &fi) {
    uint32_t j = 0;
    for (int b = 0; b < s.nd; b++) j |= (uint32_t)((idx >> s.dq[b]) & 1) << b;
    fr = s.dr[j];
    fi = s.di[j];
}

// Build the diagonal-factor table from the pending list.
__device__ void prepare_pending(Shared &s) {
    s.nd = 0;
    s.nondiag = 0;
    for (int p = 0; p < s.npend; p++) {
        const Pending &P = s.pend[p];
        const bool diag = P.m[1].re == 0 && P.m[1].im == 0 && P.m[2].re == 0 && P.m[2].im == 0;
        if (!diag) {
            s.nondiag = 1;
            continue;
        }
        s.dq[s.nd++] = p;  // temporarily the pending index
    }
    const int nd = s.nd;
    uint32_t pidx[3];
    for (int b = 0; b < nd; b++) {
        pidx[b] = s.dq[b];
        s.dq[b] = s.pend[pidx[b]].q;
    }
    for (uint32_t j = 0; j < (1u << nd); j++) {
        C2 f{1, 0};
        for (int b = 0; b < nd; b++) f = cmul(f, s.pend[pidx[b]].m[((j >> b) & 1) ? 3 : 0]);
        s.dr[j] = (float)f.re;
        s.di[j] = (float)f.im;
    }
}

// df accumulate |v|^2 (exact square via FMA, TwoSum into (hi, lo)).
__device__ __forceinline__ void acc_p2(float r, float i, float &hi, float &lo) {
    const float p0 = __fmul_rn(r, r), e0 = __fmaf_rn(r, r, -p0);
    const float p1 = __fmul_rn(i, i), e1 = __fmaf_rn(i, i, -p1);
    float err0, err1;
    float s = two_sum(hi, p0, err0);
    s = two_sum(s, p1, err1);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(err0, err1), __fadd_rn(e0, e1)));
}

// CTA reduction of per-thread tables (hi + lo in FP64) into s.J[0..cnt).
__device__ void reduce_table(Shared &s, const float *hi, const float *lo, int cnt) {
    const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
    for (int j = 0; j < cnt; j++) {
        double v = (double)hi[j] + (double)lo[j];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) s.red[warp][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < cnt) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); w++) v += s.red[w][threadIdx.x];
        s.J[threadIdx.x] = v;
    }
    __syncthreads();
}

// One op's pass for a K-qubit op (K = 1, 2, so the group's amplitudes and
// its probability table stay in registers): the pending diagonal factors,
// then the gate, accumulating |amplitude|^2 per group row into (hi, lo).
template <int K, typename T>
__device__ __forceinline__ void traj_pass(T *re, T *im, uint64_t len, const TrajOp &op, const Shared &s, float *hi,
                                          float *lo) {
    constexpr uint32_t D = 1u << K;
    uint32_t qs[K];
#pragma unroll
    for (int b = 0; b < K; b++) qs[b] = op.qs[b];
    // the op matrix is read from shared memory at each use: hoisted into
    // registers it would spill at the 64-register cap of four CTAs per SM
    const volatile float *mr = s.mr, *mi = s.mi;
    float h[D], l[D];
#pragma unroll
    for (uint32_t r = 0; r < D; r++) h[r] = l[r] = 0.f;
    const uint64_t groups = len >> K;
    for (uint64_t g = threadIdx.x; g < groups; g += blockDim.x) {
        const uint64_t base = insert_zeros(g, qs, K);
        float xr[D], xi[D];
#pragma unroll
        for (uint32_t j = 0; j < D; j++) {
            uint64_t idx = base;
#pragma unroll
            for (int b = 0; b < K; b++) idx |= (uint64_t)((j >> b) & 1) << qs[b];
            float fr, fi;
            diag_factor(s, idx, fr, fi);
            const float a = (float)re[idx], c = (float)im[idx];
            xr[j] = fr * a - fi * c;
            xi[j] = fr * c + fi * a;
        }
#pragma unroll
        for (uint32_t r = 0; r < D; r++) {
            float yr = 0.f, yi = 0.f;
#pragma unroll
            for (uint32_t c = 0; c < D; c++) {
                const float wr = mr[r * D + c], wi = mi[r * D + c];
                yr = fmaf(wr, xr[c], fmaf(-wi, xi[c], yr));
                yi = fmaf(wr, xi[c], fmaf(wi, xr[c], yi));
            }
            uint64_t idx = base;
#pragma unroll
            for (int b = 0; b < K; b++) idx |= (uint64_t)((r >> b) & 1) << qs[b];
            re[idx] = (T)yr;
            im[idx] = (T)yi;
            acc_p2(yr, yi, h[r], l[r]);
        }
    }
#pragma unroll
    for (uint32_t r = 0; r < D; r++) {
        hi[r] = h[r];
        lo[r] = l[r];
    }
}

template <typename T>
__global__ void __launch_bounds__(kTrajThreads, 4)
    k_trajectories(T *__restrict__ work, uint32_t n, const TrajOp *__restrict__ ops, int nops,
                   const double *__restrict__ mats, const uint32_t *__restrict__ fq, const uint32_t *__restrict__ fc,
                   int nfinal, TrajNoise nz, uint64_t ntraj, uint64_t seed, uint64_t *__restrict__ out,
                   int *__restrict__ err) {
    __shared__ Shared s;
    const uint64_t len = 1ull << n;
    T *re = work + (size_t)blockIdx.x * 2 * len;
    T *im = re + len;
    const int tid = threadIdx.x;
    for (uint64_t t = blockIdx.x; t < ntraj; t += gridDim.x) {
        for (uint64_t i = tid; i < len; i += blockDim.x) {
            re[i] = T(i == 0);
            im[i] = T(0);
        }
        if (tid == 0) {
            s.npend = 0;
            s.draw = 0;
            s.cl = 0;
        }
        __syncthreads();
        for (int o = 0; o < nops; o++) {
            const TrajOp op = ops[o];
            const uint32_t k = op.k, dim = 1u << k;
            const bool gate = op.kind == TOP_GATE;
            // ---- thread 0: condition, depolarizing draws, gate x Pauli string, pending factors
            if (tid == 0) {
                s.skip = 0;
                if (op.cond) {
                    const uint64_t mask = op.cond_len >= 64 ? ~0ull : ((1ull << op.cond_len) - 1);
                    s.skip = ((s.cl >> op.cond_off) & mask) != op.cond_value;
                }
            }
            __syncthreads();
            if (s.skip) {  // pending operators wait for the next op that runs
                __syncthreads();  // every thread has read s.skip before thread 0 sets it again
                continue;
            }
            if (tid == 0) {
                prepare_pending(s);
                const double pdep = gate ? (k == 1 ? nz.p[0] : nz.p[1]) : 0.0;
                uint64_t idx = 0;
                if (pdep > 0.0 && philox_f64(seed, t, s.draw++) < pdep)
                    idx = 1 + philox_range(seed, t, s.draw++, (1ull << (2 * k)) - 1);
                const double *M = mats + op.mat_off;
                // P_string . M: the Pauli string is a signed permutation, row r
                // holding its one entry in column r ^ xm (X and Y flip the bit),
                // of value prod_b v_b(r_b) (Y: -i on 0, i on 1; Z: -1 on 1)
                uint32_t xm = 0;
                for (uint32_t b = 0; b < k; b++) {
                    const uint32_t code = (uint32_t)(idx >> (2 * b)) & 3u;
                    if (code == 1 || code == 2) xm |= 1u << b;
                }
                for (uint32_t r = 0; r < dim; r++) {
                    int re_sign = 1, swap = 0;  // phase = re_sign * (swap ? i : 1)
                    for (uint32_t b = 0; b < k; b++) {
                        const uint32_t code = (uint32_t)(idx >> (2 * b)) & 3u, rb = (r >> b) & 1u;
                        if (code == 2) {  // multiply by -i (rb = 0) or i (rb = 1)
                            if (swap) re_sign = rb ? -re_sign : re_sign;  // i * i = -1, i * -i = 1
                            else re_sign = rb ? re_sign : -re_sign;
                            swap ^= 1;
                        } else if (code == 3 && rb) {
                            re_sign = -re_sign;
                        }
                    }
                    const uint32_t j = r ^ xm;
                    for (uint32_t c = 0; c < dim; c++) {
                        const float mr = (float)M[2 * (j * dim + c)], mi = (float)M[2 * (j * dim + c) + 1];
                        // (re_sign * (swap ? i : 1)) * (mr + i mi)
                        s.mr[r * dim + c] = swap ? -re_sign * mi : re_sign * mr;
                        s.mi[r * dim + c] = swap ? re_sign * mr : re_sign * mi;
                    }
                }
            }
            __syncthreads();
            if (s.nondiag) apply_nondiag_pending(re, im, n, s);
            // ---- one pass: pending diagonal factors, gate, joint table
            float hi[8] = {0}, lo[8] = {0};
            if (k == 1) {
                traj_pass<1>(re, im, len, op, s, hi, lo);
            } else if (k == 2) {
                traj_pass<2>(re, im, len, op, s, hi, lo);
            } else {  // three-qubit ops (rare): generic loop
                const uint64_t groups = len >> k;
                for (uint64_t g = tid; g < groups; g += blockDim.x) {
                    const uint64_t base = insert_zeros(g, op.qs, (int)k);
                    float xr[8], xi[8];
                    for (uint32_t j = 0; j < dim; j++) {
                        uint64_t idx = base;
                        for (uint32_t b = 0; b < k; b++) idx |= (uint64_t)((j >> b) & 1) << op.qs[b];
                        float fr, fi;
                        diag_factor(s, idx, fr, fi);
                        const float a = (float)re[idx], c = (float)im[idx];
                        xr[j] = fr * a - fi * c;
                        xi[j] = fr * c + fi * a;
                    }
                    for (uint32_t r = 0; r < dim; r++) {
                        float yr = 0.f, yi = 0.f;
                        for (uint32_t c = 0; c < dim; c++) {
                            const float wr = s.mr[r * dim + c], wi = s.mi[r * dim + c];
                            yr = fmaf(wr, xr[c], fmaf(-wi, xi[c], yr));
                            yi = fmaf(wr, xi[c], fmaf(wi, xr[c], yi));
                        }
                        uint64_t idx = base;
                        for (uint32_t b = 0; b < k; b++) idx |= (uint64_t)((r >> b) & 1) << op.qs[b];
                        re[idx] = (T)yr;
                        im[idx] = (T)yi;
                        acc_p2(yr, yi, hi[r], lo[r]);
                    }
                }
            }
            __syncthreads();
            if (tid == 0) s.npend = 0;
            reduce_table(s, hi, lo, (int)dim);
            // ---- thread 0, measure / reset: outcome from the table, collapse (and X) left pending
            if (tid == 0 && !gate) {
                const double tot = s.J[0] + s.J[1];
                const double p1 = tot > 0.0 ? s.J[1] / tot : 0.0;
                const bool one = philox_f64(seed, t, s.draw++) < p1;  // src/exec.rs:201-207
                const double sc = 1.0 / sqrt(one ? p1 : 1.0 - p1);
                Pending &P = s.pend[s.npend++];
                P.q = op.qs[0];
                for (int i = 0; i < 4; i++) P.m[i] = C2{0, 0};
                if (!one) P.m[0] = C2{(float)sc, 0};
                else if (op.kind == TOP_RESET) P.m[1] = C2{(float)sc, 0};  // X . diag(0, sc)
                else P.m[3] = C2{(float)sc, 0};
                if (op.kind == TOP_MEASURE) {
                    bool bit = one;
                    const double pr = bit ? nz.p[6] : nz.p[5];  // readout_flip (src/noise.rs:181-192)
                    if (pr > 0.0 && philox_f64(seed, t, s.draw++) < pr) bit = !bit;
                    s.cl = (s.cl & ~(1ull << op.clbit)) | ((uint64_t)bit << op.clbit);
                }
            }
            // ---- thread 0: flips and damping on the table, in the reference's order
            if (tid == 0 && gate) {
                double J[8];
                for (uint32_t j = 0; j < dim; j++) J[j] = s.J[j];
                for (uint32_t b = 0; b < k; b++) {
                    C2 M[4];
                    pauli(0, M);
                    if (nz.p[2] > 0.0 && philox_f64(seed, t, s.draw++) < nz.p[2]) {
                        C2 X[4];
                        pauli(1, X);
                        mul22(X, M, M);
                        for (uint32_t j = 0; j < dim; j++)
                            if (!((j >> b) & 1)) {
                                const double x = J[j];
                                J[j] = J[j | (1u << b)];
                                J[j | (1u << b)] = x;
                            }
                    }
                    if (nz.p[3] > 0.0 && philox_f64(seed, t, s.draw++) < nz.p[3]) {
                        C2 Z[4];
                        pauli(3, Z);
                        mul22(Z, M, M);
                    }
                    if (nz.p[4] > 0.0) {
                        const double u = philox_f64(seed, t, s.draw++);
                        double tot = 0.0, p1 = 0.0;
                        for (uint32_t j = 0; j < dim; j++) {
                            tot += J[j];
                            if ((j >> b) & 1) p1 += J[j];
                        }
                        p1 = tot > 0.0 ? p1 / tot : 0.0;
                        const double pj = nz.p[4] * p1;
                        C2 D[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
                        if (u < pj) {
                            // jump: collapse to 1 (scale 1/sqrt(P1)) then X
                            D[1] = C2{(float)(1.0 / sqrt(p1)), 0};
                            for (uint32_t j = 0; j < dim; j++)
                                if (!((j >> b) & 1)) {
                                    J[j] = J[j | (1u << b)] / p1;
                                    J[j | (1u << b)] = 0.0;
                                }
                        } else {
                            const double sc = 1.0 / sqrt(1.0 - pj);
                            const double d3 = sc * sqrt(1.0 - nz.p[4]);
                            D[0] = C2{(float)sc, 0};
                            D[3] = C2{(float)d3, 0};
                            for (uint32_t j = 0; j < dim; j++) J[j] *= ((j >> b) & 1) ? d3 * d3 : sc * sc;
                        }
                        mul22(D, M, M);
                    }
                    Pending &P = s.pend[s.npend++];
                    P.q = op.qs[b];
                    for (int i = 0; i < 4; i++) P.m[i] = M[i];
                }
            }
            __syncthreads();
        }
        // ---- final: pending operators, then one basis index from |psi|^2
        if (tid == 0) prepare_pending(s);
        __syncthreads();
        if (s.nondiag) apply_nondiag_pending(re, im, n, s);
        const uint64_t per = (len + blockDim.x - 1) / blockDim.x;
        const uint64_t i0 = tid * per, i1 = min(len, i0 + per);
        {
            float hi = 0.f, lo = 0.f;
            for (uint64_t i = i0; i < i1; i++) {
                float fr, fi;
                diag_factor(s, i, fr, fi);
                const float a = (float)re[i], c = (float)im[i];
                acc_p2(fr * a - fi * c, fr * c + fi * a, hi, lo);
            }
            s.seg[tid] = (double)hi + (double)lo;
        }
        __syncthreads();
        if (tid == 0) {
            double tot = 0.0;
            for (int i = 0; i < (int)blockDim.x; i++) tot += s.seg[i];
            double u = philox_f64(seed, t, s.draw++) * tot;
            uint64_t pick = len;
            bool found = false;
            for (int w = 0; w < (int)blockDim.x && !found; w++) {
                if (u < s.seg[w]) {
                    const uint64_t a0 = (uint64_t)w * per, a1 = min(len, a0 + per);
                    for (uint64_t i = a0; i < a1; i++) {
                        float fr, fi;
                        diag_factor(s, i, fr, fi);
                        const float a = (float)re[i], c = (float)im[i];
                        const float xr = fr * a - fi * c, xi = fr * c + fi * a;
                        const double p = (double)xr * xr + (double)xi * xi;
                        if (p > 0.0) pick = i;  // last nonzero so far
                        if (u < p) {
                            pick = i;
                            found = true;
                            break;
                        }
                        u -= p;
                    }
                    found = true;
                } else {
                    u -= s.seg[w];
                }
            }
            if (pick == len) {
                // rounding left the draw past the last segment: last index with nonzero probability
                pick = 0;
                for (uint64_t i = len; i-- > 0;) {
                    float fr, fi;
                    diag_factor(s, i, fr, fi);
                    const float a = (float)re[i], c = (float)im[i];
                    if ((fr * a - fi * c) != 0.f || (fr * c + fi * a) != 0.f) {
                        pick = i;
                        break;
                    }
                }
            }
            uint64_t cl = s.cl;
            for (int f = 0; f < nfinal; f++) {
                bool bit = (pick >> fq[f]) & 1;
                const double pr = bit ? nz.p[6] : nz.p[5];
                if (pr > 0.0 && philox_f64(seed, t, s.draw++) < pr) bit = !bit;
                cl = (cl & ~(1ull << fc[f])) | ((uint64_t)bit << fc[f]);
            }
            out[t] = cl;
        }
        __syncthreads();
    }
    (void)err;
}

}  // namespace

int launch_trajectories(zc_state *st, uint32_t n, const TrajOp *d_ops, int nops, const double *d_mats,
                        const uint32_t *d_fq, const uint32_t *d_fc, int nfinal, const TrajNoise &nz, uint64_t ntraj,
                        uint64_t seed, uint64_t *d_out, void *d_work, int ctas) {
    ProfScope ps(st, K_TRAJ, 0.0);
    st->ctr.launches++;
    if (st->prec != 32) return fail(ZC_ERR_UNSUPPORTED, "the batched trajectory engine runs f32 states");
    k_trajectories<float><<<ctas, kTrajThreads, 0, st->stream>>>((float *)d_work, n, d_ops, nops, d_mats, d_fq, d_fc,
                                                                 nfinal, nz, ntraj, seed, d_out, st->d_err);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

}  // namespace zc
