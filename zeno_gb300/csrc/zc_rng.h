// Host-side random streams with zeno's seed semantics.
//
// xoshiro256++ (Blackman & Vigna) seeded like rand_xoshiro 0.6's
// `seed_from_u64` (four SplitMix64 outputs fill the state); draws follow
// rand 0.8.5: `gen::<f64>()` = (next >> 11) * 2^-53, and `gen_range(lo..hi)`
// for u64 = widening-multiply rejection against (range << lzcnt) - 1.
// `splitmix64` is zeno's seed mixer (src/exec.rs:227-232).
#pragma once
#include <stdint.h>

namespace zc {

inline uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Xoshiro {
    uint64_t s[4];
    explicit Xoshiro(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; i++) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            s[i] = z ^ (z >> 31);
        }
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t result = rotl(s[0] + s[3], 23) + s[0];
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    double f64() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint64_t range(uint64_t lo, uint64_t hi) {
        const uint64_t r = hi - lo;
        if (r == 0) return next();
        const uint64_t zone = (r << __builtin_clzll(r)) - 1;
        for (;;) {
            const unsigned __int128 m = (unsigned __int128)next() * r;
            if ((uint64_t)m <= zone) return lo + (uint64_t)(m >> 64);
        }
    }
};

}  // namespace zc
