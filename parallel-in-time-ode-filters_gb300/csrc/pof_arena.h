// First-fit allocator of contiguous grid-point ranges of the serving
// engine's arena (pof_serve.cu).  Host-only; tested on the CPU by
// tests/arena_props.cpp.
#pragma once

#include <stdint.h>

#include <utility>
#include <vector>

namespace pof {

struct Arena {
  std::vector<std::pair<int64_t, int64_t>> free_;  // [lo, hi), sorted, coalesced
  void init(int64_t n) { free_.assign(1, {0, n}); }
  int64_t alloc(int64_t n) {
    for (size_t i = 0; i < free_.size(); ++i) {
      if (free_[i].second - free_[i].first >= n) {
        const int64_t lo = free_[i].first;
        free_[i].first += n;
        if (free_[i].first == free_[i].second) free_.erase(free_.begin() + i);
        return lo;
      }
    }
    return -1;
  }
  void release(int64_t lo, int64_t n) {
    const int64_t hi = lo + n;
    size_t i = 0;
    while (i < free_.size() && free_[i].first < lo) ++i;
    free_.insert(free_.begin() + i, {lo, hi});
    if (i + 1 < free_.size() && free_[i].second == free_[i + 1].first) {
      free_[i].second = free_[i + 1].second;
      free_.erase(free_.begin() + i + 1);
    }
    if (i > 0 && free_[i - 1].second == free_[i].first) {
      free_[i - 1].second = free_[i].second;
      free_.erase(free_.begin() + i);
    }
  }
};

}  // namespace pof
