// Host check of the sampler's host half (zeno_gb300/csrc/zc_api.cpp
// sample_route: serial prefix of the chunk masses, serial draws scaled by the
// total, ascending sort, routing of draws to chunks). Random states — with
// zero-probability stretches and chunks, f64 and f32 — get their chunk masses
// the way pass 1 forms them (serial f64 sum per 2^16-element chunk), are
// routed by the library, and the touched chunks are rescanned the way pass 2
// does (running sum from cum_before, emit while draw < sum, leftover draws to
// the chunk's last nonzero index). The indices must equal the oracle's
// sampler (src/sample.rs:29-111) at the same seed. Links the built library
// and the oracle; no GPU.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "zc_internal.h"

extern "C" {
#include "zeno_oracle.h"
}

int main() {
    std::mt19937_64 rng(8642);
    size_t cases = 0, leftovers = 0, touched = 0, draws = 0;
    for (int trial = 0; trial < 48; trial++) {
        const uint32_t n = 1 + (uint32_t)(rng() % 19);  // up to 2^19: several chunks
        const int prec = trial % 2 ? 32 : 64;
        const size_t dim = (size_t)1 << n;
        std::vector<zo_c64> amps(dim);
        std::uniform_real_distribution<double> U(-1.0, 1.0);
        const int shape = trial % 4;  // 0 dense, 1 zero stretches, 2 one nonzero block, 3 few amplitudes
        for (size_t i = 0; i < dim; i++) {
            bool zero = false;
            if (shape == 1) zero = ((i >> (n > 3 ? n - 3 : 0)) & 1) || (i % 7 == 3);
            if (shape == 2) zero = i < dim / 3 || i > dim / 3 + 40;
            if (shape == 3) zero = rng() % 97 != 0;
            amps[i] = zero ? zo_c64{0.0, 0.0} : zo_c64{U(rng), U(rng)};
        }
        amps[rng() % dim] = zo_c64{0.5, -0.25};  // a state has some probability somewhere
        zo_state *s = zo_state_new(n, prec);
        zo_load_state(s, amps.data());
        std::vector<zo_c64> sv(dim);
        zo_statevector(s, sv.data());  // the stored values (f32 states rounded)
        auto p2 = [&](size_t i) { return sv[i].re * sv[i].re + sv[i].im * sv[i].im; };
        const size_t chunk = dim < ((size_t)1 << zc::kSampleChunkLog2) ? dim : ((size_t)1 << zc::kSampleChunkLog2);
        const size_t nch = (dim + chunk - 1) / chunk;
        std::vector<double> sums(nch, 0.0);
        for (size_t c = 0; c < nch; c++)
            for (size_t i = c * chunk; i < (c + 1) * chunk && i < dim; i++) sums[c] += p2(i);
        for (uint64_t shots : {0ull, 1ull, 17ull, 4096ull}) {
            const uint64_t seed = rng();
            std::vector<uint64_t> want(shots), got(shots, ~0ull);
            zo_sample(s, shots, seed, want.data());
            zc::SampleRoute r;
            zc::sample_route(sums.data(), nch, dim, shots, seed, &r);
            if (r.us.size() != shots || (shots == 0 && !r.touched.empty())) {
                std::printf("FAIL trial %d: %zu draws, %zu touched chunks for %llu shots\n", trial, r.us.size(),
                            r.touched.size(), (unsigned long long)shots);
                return 1;
            }
            if (r.chunk_len != chunk) {
                std::printf("FAIL trial %d: chunk length %llu\n", trial, (unsigned long long)r.chunk_len);
                return 1;
            }
            for (const zc::SampleChunk &c : r.touched) {
                const size_t lo = c.chunk * chunk, hi = std::min(lo + chunk, dim);
                size_t ptr = c.s0;
                double acc = c.cum;
                for (size_t i = lo; i < hi && ptr < c.s1; i++) {
                    acc += p2(i);
                    while (ptr < c.s1 && r.us[ptr] < acc) got[ptr++] = i;
                }
                if (ptr < c.s1) {
                    size_t last_nz = hi - 1;
                    for (size_t i = hi; i-- > lo;)
                        if (p2(i) > 0.0) {
                            last_nz = i;
                            break;
                        }
                    leftovers += c.s1 - ptr;
                    while (ptr < c.s1) got[ptr++] = last_nz;
                }
                touched++;
            }
            if (got != want) {
                size_t k = 0;
                while (got[k] == want[k]) k++;
                std::printf("FAIL trial %d (n %u, f%d, %llu shots): draw %zu gives %llu, the oracle %llu\n", trial, n,
                            prec, (unsigned long long)shots, k, (unsigned long long)got[k],
                            (unsigned long long)want[k]);
                return 1;
            }
            cases++;
            draws += shots;
        }
        zo_state_free(s);
    }
    std::printf("ok cases %zu draws %zu touched %zu leftovers %zu\n", cases, draws, touched, leftovers);
    return 0;
}
