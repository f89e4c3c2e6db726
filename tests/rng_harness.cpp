// Host check of the library's seed streams (zeno_gb300/csrc/zc_rng.h) against
// published reference outputs: SplitMix64 from state 0 (Vigna's splitmix64.c)
// and xoshiro256++ from the state (1, 2, 3, 4) (the reference test of the
// rand_xoshiro crate); the seeded state is four SplitMix64 outputs.
#include <cstdio>

#include "zc_rng.h"

int main() {
    const uint64_t sm[4] = {0xe220a8397b1dcdafull, 0x6e789e6aa1b965f4ull, 0x06c45d188009454full,
                            0xf88bb8a8724c81ecull};
    const uint64_t xo[10] = {41943041ull,
                             58720359ull,
                             3588806011781223ull,
                             3591011842654386ull,
                             9228616714210784205ull,
                             9973669472204895162ull,
                             14011001112246962877ull,
                             12406186145184390807ull,
                             15849039046786891736ull,
                             10450023813501588000ull};
    uint64_t x = 0;
    for (int i = 0; i < 4; i++, x += 0x9E3779B97F4A7C15ull)
        if (zc::splitmix64(x) != sm[i]) {
            std::printf("FAIL splitmix64 %d\n", i);
            return 1;
        }
    zc::Xoshiro seeded(0);
    for (int i = 0; i < 4; i++)
        if (seeded.s[i] != sm[i]) {
            std::printf("FAIL seeding %d\n", i);
            return 1;
        }
    zc::Xoshiro r(0);
    for (int i = 0; i < 4; i++) r.s[i] = (uint64_t)(i + 1);
    for (int i = 0; i < 10; i++)
        if (r.next() != xo[i]) {
            std::printf("FAIL xoshiro256++ %d\n", i);
            return 1;
        }
    std::printf("ok\n");
    return 0;
}
