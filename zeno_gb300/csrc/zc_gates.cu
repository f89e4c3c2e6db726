// Per-op gate kernels: 1-qubit unitaries, fused k-qubit unitaries,
// diagonals, and the CX / SWAP permutations. Split-complex state (re[],
// im[] of 2^n elements), every global access a 16-byte vector where the
// index pattern allows it.
#include <algorithm>
#include <atomic>

#include "zc_arith.cuh"
#include "zc_internal.h"

namespace zc {
namespace {

constexpr int kThreads = 256;

Launch grid_for(const zc_state *st, uint64_t units) {
    uint64_t want = (units + kThreads - 1) / kThreads;
    uint64_t cap = (uint64_t)st->num_sms * 16;
    if (want > cap) want = cap;
    if (want < 1) want = 1;
    return Launch{(int)want, kThreads};
}

// ---------------------------------------------------------------- 1q

// q such that 2^q >= V: every thread owns V consecutive half indices, so
// the a-row and b-row loads are 16-byte vectors and a warp reads two
// contiguous 512-byte spans (kern_1q_scalar, src/state.rs:232-260).
template <typename T, int A>
__global__ void __launch_bounds__(kThreads) k_1q_rows(T *__restrict__ re, T *__restrict__ im, uint32_t q,
                                                      uint64_t nunits, Mat2<T> m) {
    constexpr int V = Vec<T>::N;
    MatDF md;
    if constexpr (A == AR_DF) md = df_matrix(reinterpret_cast<const double *>(m.v));
    using VT = typename Vec<T>::type;
    const uint64_t s = 1ull << q;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < nunits;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = insert_zero(u * V, q);
        VT var = *reinterpret_cast<const VT *>(re + a);
        VT vai = *reinterpret_cast<const VT *>(im + a);
        VT vbr = *reinterpret_cast<const VT *>(re + a + s);
        VT vbi = *reinterpret_cast<const VT *>(im + a + s);
        T *ar = reinterpret_cast<T *>(&var), *ai = reinterpret_cast<T *>(&vai);
        T *br = reinterpret_cast<T *>(&vbr), *bi = reinterpret_cast<T *>(&vbi);
#pragma unroll
        for (int e = 0; e < V; e++) upd2<T, A>(m, md, ar[e], ai[e], br[e], bi[e]);
        *reinterpret_cast<VT *>(re + a) = var;
        *reinterpret_cast<VT *>(im + a) = vai;
        *reinterpret_cast<VT *>(re + a + s) = vbr;
        *reinterpret_cast<VT *>(im + a + s) = vbi;
    }
}

// 2^q < V: both members of every pair sit inside one 16-byte vector.
template <typename T, int A>
__global__ void __launch_bounds__(kThreads) k_1q_inreg(T *__restrict__ re, T *__restrict__ im, uint32_t q,
                                                       uint64_t nunits, Mat2<T> m) {
    constexpr int V = Vec<T>::N;
    MatDF md;
    if constexpr (A == AR_DF) md = df_matrix(reinterpret_cast<const double *>(m.v));
    using VT = typename Vec<T>::type;
    const int s = 1 << q;
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < nunits;
         u += (uint64_t)gridDim.x * blockDim.x) {
        VT vr = *reinterpret_cast<const VT *>(re + u * V);
        VT vi = *reinterpret_cast<const VT *>(im + u * V);
        T *r = reinterpret_cast<T *>(&vr), *i = reinterpret_cast<T *>(&vi);
#pragma unroll
        for (int p = 0; p < V; p++) {
            if (p & s) continue;
            upd2<T, A>(m, md, r[p], i[p], r[p | s], i[p | s]);
        }
        *reinterpret_cast<VT *>(re + u * V) = vr;
        *reinterpret_cast<VT *>(im + u * V) = vi;
    }
}

// Scalar fallback for states shorter than two vectors.
template <typename T, int A>
__global__ void k_1q_scalar(T *re, T *im, uint32_t q, uint64_t half, Mat2<T> m) {
    MatDF md;
    if constexpr (A == AR_DF) md = df_matrix(reinterpret_cast<const double *>(m.v));
    for (uint64_t h = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; h < half;
         h += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a = insert_zero(h, q), b = a + (1ull << q);
        upd2<T, A>(m, md, re[a], im[a], re[b], im[b]);
    }
}

template <typename T, int A>
int run_1q(zc_state *st, uint32_t q, const double *m8) {
    constexpr int V = Vec<T>::N;
    Mat2<T> m;
    for (int i = 0; i < 8; i++) m.v[i] = (T)m8[i];
    T *re = (T *)st->re, *im = (T *)st->im;
    const uint64_t len = st->len;
    if (len < 2 * (uint64_t)V) {
        k_1q_scalar<T, A><<<1, 64, 0, st->stream>>>(re, im, q, len / 2, m);
    } else if ((1ull << q) >= (uint64_t)V) {
        const uint64_t nunits = len / 2 / V;
        Launch L = grid_for(st, nunits);
        k_1q_rows<T, A><<<L.blocks, L.threads, 0, st->stream>>>(re, im, q, nunits, m);
    } else {
        const uint64_t nunits = len / V;
        Launch L = grid_for(st, nunits);
        k_1q_inreg<T, A><<<L.blocks, L.threads, 0, st->stream>>>(re, im, q, nunits, m);
    }
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

// ---------------------------------------------------------------- kq

struct KqParams {
    uint64_t groups;
    uint32_t k;
    uint32_t qs[kMaxUnitaryQubits];
    uint64_t offs[1 << kMaxUnitaryQubits];  // local index j -> state-index bits
};

constexpr int kKqTile = 2048;  // amplitudes staged per CTA iteration

// Fused k-qubit unitary (kern_kq_scalar, src/state.rs:355-392): a CTA
// stages G = 2048 / 2^k groups in shared memory (gather), each thread
// forms output rows with the column sum in ascending order, then scatters.
template <typename T, bool EXACT>
__global__ void __launch_bounds__(kThreads) k_kq(T *__restrict__ re, T *__restrict__ im, KqParams p,
                                                 const T *__restrict__ mre, const T *__restrict__ mim,
                                                 uint64_t offs_hi_mask) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int dim = 1 << p.k;
    const int G = kKqTile / dim;
    const int ld = dim + 1;  // padded row: conflict-free column walks
    T *xr = reinterpret_cast<T *>(smem_raw);
    T *xi = xr + G * ld;
    T *yr = xi + G * ld;
    T *yi = yr + G * ld;
    const uint64_t ntiles = (p.groups + G - 1) / G;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t g0 = tile * G;
        for (int e = threadIdx.x; e < G * dim; e += blockDim.x) {
            const int gl = e % G, j = e / G;
            const uint64_t g = g0 + gl;
            if (g < p.groups) {
                const uint64_t idx = insert_zeros(g, p.qs, p.k) | p.offs[j];
                xr[gl * ld + j] = re[idx];
                xi[gl * ld + j] = im[idx];
            }
        }
        __syncthreads();
        for (int o = threadIdx.x; o < G * dim; o += blockDim.x) {
            const int gl = o % G, r = o / G;
            if (g0 + gl < p.groups) {
                T ar = T(0), ai = T(0);
                const T *wr = mre + (size_t)r * dim, *wi = mim + (size_t)r * dim;
                const T *x_r = xr + gl * ld, *x_i = xi + gl * ld;
                for (int c = 0; c < dim; c++) cmac<T, EXACT>(__ldg(wr + c), __ldg(wi + c), x_r[c], x_i[c], ar, ai);
                yr[gl * ld + r] = ar;
                yi[gl * ld + r] = ai;
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < G * dim; e += blockDim.x) {
            const int gl = e % G, j = e / G;
            const uint64_t g = g0 + gl;
            if (g < p.groups) {
                const uint64_t idx = insert_zeros(g, p.qs, p.k) | p.offs[j];
                re[idx] = yr[gl * ld + j];
                im[idx] = yi[gl * ld + j];
            }
        }
        __syncthreads();
    }
    (void)offs_hi_mask;
}

template <typename T, bool EXACT>
int run_kq(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_mat) {
    KqParams p{};
    p.k = k;
    p.groups = st->len >> k;
    for (uint32_t i = 0; i < k; i++) p.qs[i] = qs[i];
    const int dim = 1 << k;
    for (int j = 0; j < dim; j++) {
        uint64_t o = 0;
        for (uint32_t b = 0; b < k; b++)
            if ((j >> b) & 1) o |= 1ull << qs[b];
        p.offs[j] = o;
    }
    const int G = kKqTile / dim;
    const size_t smem = (size_t)4 * G * (dim + 1) * sizeof(T);
    static std::atomic<bool> attr_set[2] = {{false}, {false}};  // per precision, once per process
    if (!attr_set[sizeof(T) == 8]) {
        ZC_CUDA(cudaFuncSetAttribute(k_kq<T, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
        attr_set[sizeof(T) == 8] = true;
    }
    const T *mre = (const T *)dev_mat;
    const T *mim = mre + (size_t)dim * dim;
    uint64_t ntiles = (p.groups + G - 1) / G;
    int blocks = (int)std::min<uint64_t>(ntiles, (uint64_t)st->num_sms * 4);
    k_kq<T, EXACT><<<blocks, kThreads, smem, st->stream>>>((T *)st->re, (T *)st->im, p, mre, mim, 0);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

// Fused k-qubit unitary on an f64 state in fast mode: the same gather /
// row sums / scatter as k_kq, in double-float arithmetic on the FP32 pipe
// (GB300 issues FP64 ~68x slower than FP32). Amplitudes are split into
// (hi, lo) pairs as they are staged; the matrix comes pre-split as float4
// (re hi, re lo, im hi, im lo) per entry. Each output is a complex dot
// product accumulated in unnormalised pairs, renormalised every 8 terms
// and rounded back to f64 on the way out.
constexpr int kKqDfTile = 1024;  // amplitudes staged per CTA iteration

__global__ void __launch_bounds__(kThreads) k_kq_df(double *__restrict__ re, double *__restrict__ im, KqParams p,
                                                    const float4 *__restrict__ mat) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int dim = 1 << p.k;
    const int G = kKqDfTile / dim;
    const int ld = dim + 1;  // padded row: conflict-free column walks
    float2 *xr = reinterpret_cast<float2 *>(smem_raw);
    float2 *xi = xr + G * ld;
    double *yr = reinterpret_cast<double *>(xi + G * ld);
    double *yi = yr + G * ld;
    const uint64_t ntiles = (p.groups + G - 1) / G;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint64_t g0 = tile * G;
        for (int e = threadIdx.x; e < G * dim; e += blockDim.x) {
            const int gl = e % G, j = e / G;
            const uint64_t g = g0 + gl;
            if (g < p.groups) {
                const uint64_t idx = insert_zeros(g, p.qs, p.k) | p.offs[j];
                xr[gl * ld + j] = df_from_f64(re[idx]);
                xi[gl * ld + j] = df_from_f64(im[idx]);
            }
        }
        __syncthreads();
        for (int o = threadIdx.x; o < G * dim; o += blockDim.x) {
            const int gl = o % G, r = o / G;
            if (g0 + gl < p.groups) {
                float2 ar = make_float2(0.f, 0.f), ai = make_float2(0.f, 0.f);
                const float4 *w = mat + (size_t)r * dim;
                const float2 *x_r = xr + gl * ld, *x_i = xi + gl * ld;
                for (int c = 0; c < dim; c++) {
                    const float4 wc = __ldg(w + c);
                    const float2 wr = make_float2(wc.x, wc.y), wi = make_float2(wc.z, wc.w);
                    const float2 vr = x_r[c], vi = x_i[c];
                    // (ar, ai) += (wr + i wi)(vr + i vi)
                    ar = df_axpy_u(ar, wr, vr);
                    ar = df_axpy_u(ar, df_neg(wi), vi);
                    ai = df_axpy_u(ai, wr, vi);
                    ai = df_axpy_u(ai, wi, vr);
                    if ((c & 7) == 7) {
                        ar = df_renorm(ar);
                        ai = df_renorm(ai);
                    }
                }
                yr[gl * ld + r] = df_to_f64(df_renorm(ar));
                yi[gl * ld + r] = df_to_f64(df_renorm(ai));
            }
        }
        __syncthreads();
        for (int e = threadIdx.x; e < G * dim; e += blockDim.x) {
            const int gl = e % G, j = e / G;
            const uint64_t g = g0 + gl;
            if (g < p.groups) {
                const uint64_t idx = insert_zeros(g, p.qs, p.k) | p.offs[j];
                re[idx] = yr[gl * ld + j];
                im[idx] = yi[gl * ld + j];
            }
        }
        __syncthreads();
    }
}

int run_kq_df(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_mat) {
    KqParams p{};
    p.k = k;
    p.groups = st->len >> k;
    for (uint32_t i = 0; i < k; i++) p.qs[i] = qs[i];
    const int dim = 1 << k;
    for (int j = 0; j < dim; j++) {
        uint64_t o = 0;
        for (uint32_t b = 0; b < k; b++)
            if ((j >> b) & 1) o |= 1ull << qs[b];
        p.offs[j] = o;
    }
    const int G = kKqDfTile / dim;
    const size_t smem = (size_t)G * (dim + 1) * (2 * sizeof(float2) + 2 * sizeof(double));
    static std::atomic<bool> attr_set{false};  // once per process
    if (!attr_set) {
        ZC_CUDA(cudaFuncSetAttribute(k_kq_df, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
        attr_set = true;
    }
    const uint64_t ntiles = (p.groups + G - 1) / G;
    // 32-41 KiB of shared memory and 32 registers per thread: five CTAs fit an
    // SM (ncu at 26q, k = 5, with three: 72% issue, 31% warps active)
    const int blocks = (int)std::min<uint64_t>(ntiles, (uint64_t)st->num_sms * 5);
    k_kq_df<<<blocks, kThreads, smem, st->stream>>>((double *)st->re, (double *)st->im, p,
                                                    (const float4 *)dev_mat);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

// ---------------------------------------------------------------- diagonals

// 1-qubit diagonal (kern_diag1_scalar, src/state.rs:498-527).
template <typename T, int A>
__global__ void __launch_bounds__(kThreads) k_diag1(T *__restrict__ re, T *__restrict__ im, uint32_t q,
                                                    uint64_t nunits, T d0r, T d0i, T d1r, T d1i) {
    constexpr int V = Vec<T>::N;
    using VT = typename Vec<T>::type;
    float2 e0r{}, e0i{}, e1r{}, e1i{};
    if constexpr (A == AR_DF) {
        e0r = df_from_f64(d0r), e0i = df_from_f64(d0i), e1r = df_from_f64(d1r), e1i = df_from_f64(d1i);
    }
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < nunits;
         u += (uint64_t)gridDim.x * blockDim.x) {
        VT vr = *reinterpret_cast<const VT *>(re + u * V);
        VT vi = *reinterpret_cast<const VT *>(im + u * V);
        T *r = reinterpret_cast<T *>(&vr), *i = reinterpret_cast<T *>(&vi);
#pragma unroll
        for (int e = 0; e < V; e++) {
            const bool one = ((u * V + e) >> q) & 1;
            scale2<T, A>(one ? d1r : d0r, one ? d1i : d0i, one ? e1r : e0r, one ? e1i : e0i, r[e], i[e]);
        }
        *reinterpret_cast<VT *>(re + u * V) = vr;
        *reinterpret_cast<VT *>(im + u * V) = vi;
    }
}

template <typename T, int A>
__global__ void k_diag1_scalar(T *re, T *im, uint32_t q, uint64_t len, T d0r, T d0i, T d1r, T d1i) {
    for (uint64_t i = threadIdx.x; i < len; i += blockDim.x) {
        const bool one = (i >> q) & 1;
        cscale<T, A == AR_EXACT>(one ? d1r : d0r, one ? d1i : d0i, re[i], im[i]);
    }
}

struct DiagParams {
    uint32_t k;
    uint32_t qs[kMaxDiagQubits];
};

// k-qubit diagonal (kern_diagk_scalar, src/state.rs:577-596): table in
// shared memory, j gathered from the index bits at qs.
template <typename T, int A>
__global__ void __launch_bounds__(kThreads) k_diagk(T *__restrict__ re, T *__restrict__ im, uint64_t nunits,
                                                    DiagParams p, const T *__restrict__ dre,
                                                    const T *__restrict__ dim_) {
    constexpr int V = Vec<T>::N;
    using VT = typename Vec<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int dim = 1 << p.k;
    T *tr = reinterpret_cast<T *>(smem_raw);
    T *ti = tr + dim;
    for (int j = threadIdx.x; j < dim; j += blockDim.x) {
        tr[j] = dre[j];
        ti[j] = dim_[j];
    }
    __syncthreads();
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < nunits;
         u += (uint64_t)gridDim.x * blockDim.x) {
        VT vr = *reinterpret_cast<const VT *>(re + u * V);
        VT vi = *reinterpret_cast<const VT *>(im + u * V);
        T *r = reinterpret_cast<T *>(&vr), *i = reinterpret_cast<T *>(&vi);
#pragma unroll
        for (int e = 0; e < V; e++) {
            const uint64_t idx = u * V + e;
            uint32_t j = 0;
            for (uint32_t b = 0; b < p.k; b++) j |= (uint32_t)((idx >> p.qs[b]) & 1) << b;
            if constexpr (A == AR_DF)
                scale2<T, A>(tr[j], ti[j], df_from_f64(tr[j]), df_from_f64(ti[j]), r[e], i[e]);
            else
                cscale<T, A == AR_EXACT>(tr[j], ti[j], r[e], i[e]);
        }
        *reinterpret_cast<VT *>(re + u * V) = vr;
        *reinterpret_cast<VT *>(im + u * V) = vi;
    }
}

template <typename T, int A>
__global__ void k_diag_scalar(T *re, T *im, uint64_t len, DiagParams p, const T *dre, const T *dim_) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < len;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t j = 0;
        for (uint32_t b = 0; b < p.k; b++) j |= (uint32_t)((i >> p.qs[b]) & 1) << b;
        cscale<T, A == AR_EXACT>(dre[j], dim_[j], re[i], im[i]);
    }
}

template <typename T, int A>
int run_diag1(zc_state *st, uint32_t q, const double *d4) {
    constexpr int V = Vec<T>::N;
    T *re = (T *)st->re, *im = (T *)st->im;
    if (st->len < (uint64_t)V) {
        k_diag1_scalar<T, A><<<1, 32, 0, st->stream>>>(re, im, q, st->len, (T)d4[0], (T)d4[1], (T)d4[2],
                                                           (T)d4[3]);
        ZC_CUDA(cudaGetLastError());
        return ZC_OK;
    }
    const uint64_t nunits = st->len / V;
    Launch L = grid_for(st, nunits);
    k_diag1<T, A><<<L.blocks, L.threads, 0, st->stream>>>(re, im, q, nunits, (T)d4[0], (T)d4[1], (T)d4[2],
                                                               (T)d4[3]);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

template <typename T, int A>
int run_diagk(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_diag) {
    constexpr int V = Vec<T>::N;
    DiagParams p{};
    p.k = k;
    for (uint32_t i = 0; i < k; i++) p.qs[i] = qs[i];
    const int dim = 1 << k;
    const T *dre = (const T *)dev_diag, *dim_ = dre + dim;
    T *re = (T *)st->re, *im = (T *)st->im;
    if (st->len < (uint64_t)V) {
        k_diag_scalar<T, A><<<1, 64, 0, st->stream>>>(re, im, st->len, p, dre, dim_);
    } else {
        static std::atomic<bool> attr_set[2] = {{false}, {false}};  // per precision, once per process
        if (!attr_set[sizeof(T) == 8]) {
            ZC_CUDA(cudaFuncSetAttribute(k_diagk<T, A>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
            attr_set[sizeof(T) == 8] = true;
        }
        const uint64_t nunits = st->len / V;
        Launch L = grid_for(st, nunits);
        k_diagk<T, A><<<L.blocks, L.threads, 2 * dim * sizeof(T), st->stream>>>(re, im, nunits, p, dre, dim_);
    }
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

// ---------------------------------------------------------------- permutations

// Swap element pairs (base | x, base | y) over all bases with zeros at
// positions lo < hi. CX: x = 1<<c, y = x | 1<<t (apply_cx,
// src/state.rs:397-417). SWAP(a, b): x = 1<<a, y = 1<<b. When lo >= log2 V
// a thread moves V consecutive bases as one vector.
template <typename T, int V>
__global__ void __launch_bounds__(kThreads) k_pair_swap(T *__restrict__ re, T *__restrict__ im, uint32_t lo,
                                                        uint32_t hi, uint64_t x, uint64_t y, uint64_t nunits) {
    using VT = typename std::conditional<V == 1, T, typename Vec<T>::type>::type;
    const uint32_t qs[2] = {lo, hi};
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < nunits;
         u += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t base = insert_zeros(u * V, qs, 2);
        VT *rx = reinterpret_cast<VT *>(re + (base | x)), *ry = reinterpret_cast<VT *>(re + (base | y));
        VT *ix = reinterpret_cast<VT *>(im + (base | x)), *iy = reinterpret_cast<VT *>(im + (base | y));
        VT a = *rx, b = *ry;
        *rx = b;
        *ry = a;
        a = *ix;
        b = *iy;
        *ix = b;
        *iy = a;
    }
}

template <typename T>
int run_pair_swap(zc_state *st, uint32_t lo, uint32_t hi, uint64_t x, uint64_t y) {
    constexpr int V = Vec<T>::N;
    const uint64_t groups = st->len >> 2;
    T *re = (T *)st->re, *im = (T *)st->im;
    if ((1ull << lo) >= (uint64_t)V && groups >= (uint64_t)V) {
        const uint64_t nunits = groups / V;
        Launch L = grid_for(st, nunits);
        k_pair_swap<T, V><<<L.blocks, L.threads, 0, st->stream>>>(re, im, lo, hi, x, y, nunits);
    } else {
        Launch L = grid_for(st, groups);
        k_pair_swap<T, 1><<<L.blocks, L.threads, 0, st->stream>>>(re, im, lo, hi, x, y, groups);
    }
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

// ---------------------------------------------------------------- collapse / reset

// collapse (src/state.rs:630-661): keep side scaled by T(1/sqrt(p)),
// other side zeroed.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_collapse(T *__restrict__ re, T *__restrict__ im, uint32_t q,
                                                       uint64_t half, int outcome, T scale) {
    const uint64_t s = 1ull << q;
    for (uint64_t h = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; h < half;
         h += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t a0 = insert_zero(h, q);
        const uint64_t keep = outcome ? a0 + s : a0, zero = outcome ? a0 : a0 + s;
        re[keep] = rmul(re[keep], scale);
        im[keep] = rmul(im[keep], scale);
        re[zero] = T(0);
        im[zero] = T(0);
    }
}

template <typename T>
__global__ void k_set_one(T *re) {
    re[0] = T(1);
}

}  // namespace

int launch_1q(zc_state *st, uint32_t q, const double *m8, bool exact) {
    ProfScope ps(st, K_1Q, 2.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * (st->prec / 8) * 2;
    if (st->prec == 64) return exact ? run_1q<double, AR_EXACT>(st, q, m8) : run_1q<double, AR_DF>(st, q, m8);
    return exact ? run_1q<float, AR_EXACT>(st, q, m8) : run_1q<float, AR_FMA>(st, q, m8);
}

int launch_kq(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_mat, bool exact) {
    ProfScope ps(st, K_KQ, 2.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * (st->prec / 8) * 2;
    if (st->prec == 64)
        return exact ? run_kq<double, true>(st, qs, k, dev_mat) : run_kq<double, false>(st, qs, k, dev_mat);
    return exact ? run_kq<float, true>(st, qs, k, dev_mat) : run_kq<float, false>(st, qs, k, dev_mat);
}

int launch_kq_df(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_mat_df) {
    ProfScope ps(st, K_KQ, 2.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * (st->prec / 8) * 2;
    if (st->prec != 64) return fail(ZC_ERR_INVALID, "double-float dense blocks need an f64 state");
    return run_kq_df(st, qs, k, dev_mat_df);
}

int launch_diag1(zc_state *st, uint32_t q, const double *d4, bool exact) {
    ProfScope ps(st, K_DIAG1, 2.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * (st->prec / 8) * 2;
    if (st->prec == 64) return exact ? run_diag1<double, AR_EXACT>(st, q, d4) : run_diag1<double, AR_DF>(st, q, d4);
    return exact ? run_diag1<float, AR_EXACT>(st, q, d4) : run_diag1<float, AR_FMA>(st, q, d4);
}

int launch_diagk(zc_state *st, const uint32_t *qs, uint32_t k, const void *dev_diag, bool exact) {
    ProfScope ps(st, K_DIAGK, 2.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += 2 * st->len * (st->prec / 8) * 2;
    if (st->prec == 64)
        return exact ? run_diagk<double, AR_EXACT>(st, qs, k, dev_diag) : run_diagk<double, AR_DF>(st, qs, k, dev_diag);
    return exact ? run_diagk<float, AR_EXACT>(st, qs, k, dev_diag) : run_diagk<float, AR_FMA>(st, qs, k, dev_diag);
}

int launch_cx(zc_state *st, uint32_t c, uint32_t t) {
    ProfScope ps(st, K_CX, 1.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += st->len * (st->prec / 8) * 2;  // half the amplitudes, read + write
    const uint32_t lo = std::min(c, t), hi = std::max(c, t);
    const uint64_t x = 1ull << c, y = x | (1ull << t);
    return st->prec == 64 ? run_pair_swap<double>(st, lo, hi, x, y) : run_pair_swap<float>(st, lo, hi, x, y);
}

int launch_swap(zc_state *st, uint32_t a, uint32_t b) {
    ProfScope ps(st, K_SWAP, 1.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    st->ctr.sweeps++;
    st->ctr.bytes_moved += st->len * (st->prec / 8) * 2;
    const uint32_t lo = std::min(a, b), hi = std::max(a, b);
    const uint64_t x = 1ull << lo, y = 1ull << hi;
    return st->prec == 64 ? run_pair_swap<double>(st, lo, hi, x, y) : run_pair_swap<float>(st, lo, hi, x, y);
}

int launch_collapse(zc_state *st, uint32_t q, int outcome, double scale64) {
    ProfScope ps(st, K_COLLAPSE, 2.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    const uint64_t half = st->len / 2;
    Launch L = grid_for(st, half);
    if (st->prec == 64)
        k_collapse<double><<<L.blocks, L.threads, 0, st->stream>>>((double *)st->re, (double *)st->im, q, half,
                                                                   outcome, scale64);
    else
        k_collapse<float><<<L.blocks, L.threads, 0, st->stream>>>((float *)st->re, (float *)st->im, q, half,
                                                                  outcome, (float)scale64);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

int launch_reset(zc_state *st) {
    ProfScope ps(st, K_RESET, 1.0 * st->len * (st->prec / 8) * 2);
    st->ctr.launches++;
    const size_t bytes = st->len * (st->prec / 8);
    ZC_CUDA(cudaMemsetAsync(st->re, 0, bytes, st->stream));
    ZC_CUDA(cudaMemsetAsync(st->im, 0, bytes, st->stream));
    if (st->prec == 64)
        k_set_one<double><<<1, 1, 0, st->stream>>>((double *)st->re);
    else
        k_set_one<float><<<1, 1, 0, st->stream>>>((float *)st->re);
    ZC_CUDA(cudaGetLastError());
    return ZC_OK;
}

}  // namespace zc
