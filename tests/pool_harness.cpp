// Host check of the serving engine's pool allocator (zeno_gb300/csrc/zc_pool.h)
// and of its admission rule (zc_serve.cpp, zc_server_step: FIFO, admitted
// while a slot is free and the state fits). Random request streams of
// 256-byte-rounded state sizes are admitted, run for a random number of
// steps and released; after every call the free list must be sorted,
// coalesced and disjoint from the live blocks, together covering the pool,
// and every allocation must be the first fit. Every request must finish.
#include <algorithm>
#include <cstdio>
#include <deque>
#include <random>
#include <vector>

#include "zc_pool.h"

namespace {

struct Live {
    size_t off, bytes;
    int steps_left;
};

bool check(const zc::PoolFreeList &pl, const std::vector<Live> &live, size_t pool, const char **why) {
    const auto &fl = pl.blocks();
    size_t covered = 0;
    for (size_t i = 0; i < fl.size(); i++) {
        if (fl[i].second == 0) return *why = "empty free block", false;
        if (fl[i].first + fl[i].second > pool) return *why = "free block past the pool", false;
        if (i && fl[i - 1].first + fl[i - 1].second >= fl[i].first)
            return *why = fl[i - 1].first + fl[i - 1].second == fl[i].first ? "free blocks not merged"
                                                                              : "free blocks overlap",
                   false;
        covered += fl[i].second;
    }
    std::vector<std::pair<size_t, size_t>> all(fl.begin(), fl.end());
    for (const Live &l : live) {
        all.push_back({l.off, l.bytes});
        covered += l.bytes;
    }
    std::sort(all.begin(), all.end());
    for (size_t i = 1; i < all.size(); i++)
        if (all[i - 1].first + all[i - 1].second > all[i].first) return *why = "blocks overlap", false;
    if (covered != pool) return *why = "free + live != pool", false;
    return true;
}

}  // namespace

int main() {
    std::mt19937_64 rng(1357);
    size_t allocs = 0, fails = 0, merged_to_one = 0, finished_total = 0;
    for (int trial = 0; trial < 400; trial++) {
        const size_t pool = (size_t)256 << (8 + rng() % 8);  // 64 KiB .. 8 MiB
        const uint32_t max_slots = 1 + (uint32_t)(rng() % 12);
        zc::PoolFreeList pl;
        pl.reset(pool);
        std::deque<size_t> pending;
        std::vector<Live> live;
        const int nreq = 20 + (int)(rng() % 60);
        int submitted = 0, finished = 0, steps = 0;
        const char *why = nullptr;
        while (finished < nreq) {
            if (++steps > 100000) {
                std::printf("FAIL trial %d: requests never finish\n", trial);
                return 1;
            }
            // arrivals: state sizes of 256 B x 2^k, at most the whole pool
            for (int a = (int)(rng() % 3); a > 0 && submitted < nreq; a--, submitted++) {
                size_t bytes = (size_t)256 << (rng() % 12);
                if (bytes > pool) bytes = pool;
                pending.push_back(bytes);
            }
            // admission: FIFO while a slot is free and the head fits
            while (!pending.empty() && live.size() < max_slots) {
                const size_t bytes = pending.front();
                size_t first_fit = (size_t)-1;
                for (const auto &f : pl.blocks())
                    if (f.second >= bytes) {
                        first_fit = f.first;
                        break;
                    }
                size_t off = 0;
                const bool ok = pl.alloc(bytes, &off);
                if (ok != (first_fit != (size_t)-1) || (ok && off != first_fit) || (ok && off % 256)) {
                    std::printf("FAIL trial %d: allocation of %zu at %zu (first fit %zu)\n", trial, bytes, off,
                                first_fit);
                    return 1;
                }
                if (!ok) {
                    fails++;
                    break;
                }
                allocs++;
                pending.pop_front();
                live.push_back({off, bytes, 1 + (int)(rng() % 4)});
                if (!check(pl, live, pool, &why)) {
                    std::printf("FAIL trial %d after alloc: %s\n", trial, why);
                    return 1;
                }
            }
            // one step of work; finished requests give their blocks back
            for (size_t i = 0; i < live.size();) {
                if (--live[i].steps_left == 0) {
                    pl.release(live[i].off, live[i].bytes);
                    live.erase(live.begin() + (long)i);
                    finished++;
                    if (!check(pl, live, pool, &why)) {
                        std::printf("FAIL trial %d after release: %s\n", trial, why);
                        return 1;
                    }
                } else {
                    i++;
                }
            }
        }
        finished_total += (size_t)finished;
        if (pl.blocks().size() == 1 && pl.blocks()[0].first == 0 && pl.blocks()[0].second == pool &&
            pl.free_bytes() == pool)
            merged_to_one++;
        else {
            std::printf("FAIL trial %d: empty pool is not one block\n", trial);
            return 1;
        }
    }
    std::printf("ok allocs %zu waits %zu finished %zu empty_pools_whole %zu\n", allocs, fails, finished_total,
                merged_to_one);
    return 0;
}
