// Host check of the trajectory engine's generator (zeno_gb300/csrc/zc_philox.h):
// Philox4x32-10 against the known-answer vectors published with the Random123
// library (counter, key -> output), then the f64 and range conversions.
#include <cmath>
#include <cstdio>

#include "zc_philox.h"

int main() {
    struct Kat {
        zc::PhiloxU4 ctr;
        uint32_t k0, k1;
        zc::PhiloxU4 out;
    };
    const Kat kats[] = {
        {{0u, 0u, 0u, 0u}, 0u, 0u, {0x6627e8d5u, 0xe169c58du, 0xbc57ac4cu, 0x9b00dbd8u}},
        {{0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu}, 0xffffffffu, 0xffffffffu,
         {0x408f276du, 0x41c83b0eu, 0xa20bc7c6u, 0x6d5451fdu}},
        {{0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u}, 0xa4093822u, 0x299f31d0u,
         {0xd16cfe09u, 0x94fdccebu, 0x5001e420u, 0x24126ea1u}},
    };
    for (const Kat &k : kats) {
        const zc::PhiloxU4 r = zc::philox4x32_10(k.ctr, k.k0, k.k1);
        if (r.x != k.out.x || r.y != k.out.y || r.z != k.out.z || r.w != k.out.w) {
            std::printf("FAIL kat %08x %08x %08x %08x\n", r.x, r.y, r.z, r.w);
            return 1;
        }
    }
    // counter layout: block i of trajectory t is counter (i lo, i hi, t lo, t hi), key = seed
    const uint64_t seed = 0x299f31d0a4093822ull, t = 0x0370734413198a2eull, i = 0x85a308d3243f6a88ull;
    const zc::PhiloxU4 b = zc::philox_block(seed, t, i);
    if (b.x != 0xd16cfe09u || b.w != 0x24126ea1u) {
        std::printf("FAIL block layout\n");
        return 1;
    }
    // conversions: f64 in [0, 1) with mean 1/2; range in [0, n) with uniform bins
    const int N = 1 << 20;
    double sum = 0.0, lo = 1.0, hi = 0.0;
    long bins[7] = {0};
    for (int d = 0; d < N; d++) {
        const double u = zc::philox_f64(42, 7, (uint64_t)d);
        if (!(u >= 0.0 && u < 1.0)) {
            std::printf("FAIL f64 %.17g\n", u);
            return 1;
        }
        sum += u;
        lo = std::fmin(lo, u);
        hi = std::fmax(hi, u);
        const uint64_t r = zc::philox_range(42, 8, (uint64_t)d, 7);
        if (r >= 7) {
            std::printf("FAIL range %llu\n", (unsigned long long)r);
            return 1;
        }
        bins[r]++;
    }
    const double mean = sum / N, sd = std::sqrt(1.0 / 12.0 / N);
    if (std::fabs(mean - 0.5) > 6 * sd || lo > 1e-4 || hi < 1 - 1e-4) {
        std::printf("FAIL f64 mean %.6f lo %.3g hi %.6f\n", mean, lo, hi);
        return 1;
    }
    const double p = 1.0 / 7, sb = std::sqrt(N * p * (1 - p));
    for (long c : bins)
        if (std::fabs((double)c - N * p) > 6 * sb) {
            std::printf("FAIL range bin %ld\n", c);
            return 1;
        }
    std::printf("ok kats 3 mean %.6f\n", mean);
    return 0;
}
