#pragma once
// Offsets in the serving engine's HBM pool: first-fit allocation over a free
// list kept sorted by offset, each released block merged with its free
// neighbours, so that a pool with nothing allocated is one block again and a
// request that fits the pool is admitted once enough requests before it
// have finished.
#include <stddef.h>

#include <algorithm>
#include <utility>
#include <vector>

namespace zc {

class PoolFreeList {
   public:
    void reset(size_t bytes) {
        free_.clear();
        if (bytes) free_.push_back({0, bytes});
    }

    // The lowest free block that holds `bytes` gives its first bytes.
    bool alloc(size_t bytes, size_t *off) {
        for (size_t i = 0; i < free_.size(); i++) {
            auto &f = free_[i];
            if (f.second >= bytes) {
                *off = f.first;
                f.first += bytes;
                f.second -= bytes;
                if (f.second == 0) free_.erase(free_.begin() + (long)i);
                return true;
            }
        }
        return false;
    }

    void release(size_t off, size_t bytes) {
        auto it = std::lower_bound(free_.begin(), free_.end(), std::make_pair(off, (size_t)0));
        it = free_.insert(it, {off, bytes});
        size_t i = (size_t)(it - free_.begin());
        if (i + 1 < free_.size() && free_[i].first + free_[i].second == free_[i + 1].first) {
            free_[i].second += free_[i + 1].second;
            free_.erase(free_.begin() + (long)i + 1);
        }
        if (i > 0 && free_[i - 1].first + free_[i - 1].second == free_[i].first) {
            free_[i - 1].second += free_[i].second;
            free_.erase(free_.begin() + (long)i);
        }
    }

    size_t free_bytes() const {
        size_t b = 0;
        for (const auto &f : free_) b += f.second;
        return b;
    }

    // (offset, length) of every free block, ascending
    const std::vector<std::pair<size_t, size_t>> &blocks() const { return free_; }

   private:
    std::vector<std::pair<size_t, size_t>> free_;
};

}  // namespace zc
