"""Seeded random streams used by the workload generators and the executor.

xoshiro256++ (Blackman & Vigna) seeded the way rand_xoshiro 0.6's
`seed_from_u64` does it (four SplitMix64 outputs fill the state), with the
draws of rand 0.8.5: `gen::<f64>()` = (next >> 11) * 2^-53 and
`gen_range(lo..hi)` for u64 = widening-multiply rejection against the
zone `(range << lzcnt(range)) - 1`.  `splitmix64` is zeno's seed mixer
(src/exec.rs:227-232).
"""

M64 = (1 << 64) - 1


def splitmix64(x: int) -> int:
    z = (x + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def _rotl(x: int, k: int) -> int:
    return ((x << k) | (x >> (64 - k))) & M64


class Xoshiro256pp:
    __slots__ = ("s",)

    def __init__(self, seed: int):
        x = seed & M64
        s = []
        for _ in range(4):
            x = (x + 0x9E3779B97F4A7C15) & M64
            z = x
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
            s.append(z ^ (z >> 31))
        self.s = s

    def next_u64(self) -> int:
        s = self.s
        result = (_rotl((s[0] + s[3]) & M64, 23) + s[0]) & M64
        t = (s[1] << 17) & M64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = _rotl(s[3], 45)
        return result

    def f64(self) -> float:
        return float(self.next_u64() >> 11) * (1.0 / 9007199254740992.0)

    def range(self, lo: int, hi: int) -> int:
        """Uniform integer in [lo, hi)."""
        rng = (hi - lo) & M64
        if rng == 0:
            return self.next_u64()
        lz = 64 - rng.bit_length()
        zone = ((rng << lz) & M64) - 1
        while True:
            v = self.next_u64()
            m = v * rng
            if (m & M64) <= zone:
                return lo + (m >> 64)
