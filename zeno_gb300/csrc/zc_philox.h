#pragma once
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11): ten rounds of two
// 32x32->64 multiplies with the published multipliers and Weyl key
// increments. Host and device: the trajectory engine draws on the device,
// the known-answer test runs on the host.
#include <stdint.h>

#ifdef __CUDACC__
#define ZC_PHILOX_HD __host__ __device__ __forceinline__
#else
#define ZC_PHILOX_HD inline
#endif

namespace zc {

struct PhiloxU4 {
    uint32_t x, y, z, w;
};

ZC_PHILOX_HD PhiloxU4 philox4x32_10(PhiloxU4 c, uint32_t k0, uint32_t k1) {
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        c = PhiloxU4{(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

// Block `i` of trajectory `t`'s stream: counter (i, t), key = seed.
ZC_PHILOX_HD PhiloxU4 philox_block(uint64_t seed, uint64_t t, uint64_t i) {
    return philox4x32_10(PhiloxU4{(uint32_t)i, (uint32_t)(i >> 32), (uint32_t)t, (uint32_t)(t >> 32)},
                         (uint32_t)seed, (uint32_t)(seed >> 32));
}

// Uniform f64 in [0, 1): 53 bits (27 from x, 26 from y) times 2^-53.
ZC_PHILOX_HD double philox_f64(uint64_t seed, uint64_t t, uint64_t i) {
    const PhiloxU4 r = philox_block(seed, t, i);
    const uint64_t bits = ((uint64_t)(r.x >> 5) << 26) | (uint64_t)(r.y >> 6);
    return (double)bits * (1.0 / 9007199254740992.0);
}

// Integer in [0, n): the 64 bits (z, w) scaled by n (multiply-shift; bias
// below n / 2^64).
ZC_PHILOX_HD uint64_t philox_range(uint64_t seed, uint64_t t, uint64_t i, uint64_t n) {
    const PhiloxU4 r = philox_block(seed, t, i);
    const uint64_t v = ((uint64_t)r.z << 32) | r.w;
    return (uint64_t)(((unsigned __int128)v * n) >> 64);
}

}  // namespace zc
