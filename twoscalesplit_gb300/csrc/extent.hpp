// extent.hpp -- first-fit allocator of page-aligned extents, the bookkeeping of a
// scene pool's resources (low-res slots, grid cells, wall particles).
//
// Host-only C++, no CUDA: each resource of a pool is one linear array on the
// device, and a scene owns one contiguous run of whole pages of it (a scene's slot
// ids, its grid's cells and its walls must be contiguous, because the kernels
// address them as base + local index).  Freed runs merge with their neighbours,
// and the lowest-addressed run that fits is taken, which keeps the occupied part
// of each array packed towards zero: the grid scan and the other kernels whose
// cost follows the occupied range (the high-water mark) stay cheap.
#pragma once
#include <cstdint>
#include <iterator>
#include <map>

namespace tss {

class ExtentSet {
  public:
    ExtentSet() = default;
    ExtentSet(int64_t capacity, int64_t page) { reset(capacity, page); }

    void reset(int64_t capacity, int64_t page) {
        page_ = page > 0 ? page : 1;
        cap_ = capacity > 0 ? (capacity / page_) * page_ : 0;
        free_.clear();
        used_.clear();
        if (cap_ > 0) free_[0] = cap_;
        free_total_ = cap_;
    }

    int64_t pages(int64_t n) const { return (n + page_ - 1) / page_; }
    int64_t rounded(int64_t n) const { return pages(n) * page_; }
    int64_t capacity() const { return cap_; }
    int64_t free_units() const { return free_total_; }
    int64_t page() const { return page_; }

    // First fit of n units (rounded up to whole pages; n == 0 takes nothing and
    // returns the current high-water mark as its address).
    bool alloc(int64_t n, int64_t* at) {
        if (n < 0) return false;
        if (n == 0) {
            *at = high_water();
            return true;
        }
        const int64_t len = rounded(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < len) continue;
            const int64_t start = it->first;
            const int64_t rest = it->second - len;
            free_.erase(it);
            if (rest > 0) free_[start + len] = rest;
            used_[start] = len;
            free_total_ -= len;
            *at = start;
            return true;
        }
        return false;
    }

    // Would n units fit now / ever (in an empty set)?
    bool fits_now(int64_t n) const {
        if (n <= 0) return true;
        const int64_t len = rounded(n);
        for (const auto& f : free_)
            if (f.second >= len) return true;
        return false;
    }
    bool fits_ever(int64_t n) const { return n <= 0 || rounded(n) <= cap_; }

    // Release the run that alloc() returned at `at`; false if there is none.
    bool release(int64_t at) {
        auto u = used_.find(at);
        if (u == used_.end()) return false;
        int64_t start = at, len = u->second;
        used_.erase(u);
        free_total_ += len;
        auto next = free_.lower_bound(start);
        if (next != free_.end() && next->first == start + len) {  // merge with the run after
            len += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {  // merge with the run before
            auto prev = std::prev(next);
            if (prev->first + prev->second == start) {
                start = prev->first;
                len += prev->second;
                free_.erase(prev);
            }
        }
        free_[start] = len;
        return true;
    }

    // End of the last allocated run (0 when nothing is allocated).
    int64_t high_water() const {
        if (used_.empty()) return 0;
        auto last = std::prev(used_.end());
        return last->first + last->second;
    }

    // Length of the run allocated at `at` (0 if none).
    int64_t length(int64_t at) const {
        auto u = used_.find(at);
        return u == used_.end() ? 0 : u->second;
    }

  private:
    int64_t cap_ = 0, page_ = 1, free_total_ = 0;
    std::map<int64_t, int64_t> free_;  // start -> length
    std::map<int64_t, int64_t> used_;  // start -> length
};

}  // namespace tss
