// Property checks of the serving engine's first-fit arena (pof_arena.h),
// compiled with the host compiler alone and run by tests/test_plan_cpu.py.
// Random sequences of allocations and releases are mirrored in a byte map of
// the arena; after every operation the free list must be sorted, coalesced
// (no two adjacent ranges touch) and exactly the unowned grid points; an
// allocation must return the lowest free range that fits (first fit) or -1
// when none does.  Prints "ok <cases>" and exits 0, or the first failure and
// exits 1.
#include <stdio.h>
#include <stdlib.h>

#include <random>
#include <utility>
#include <vector>

#include "pof_arena.h"

namespace {

bool check_free_list(const pof::Arena& a, const std::vector<int>& owner, const char** why) {
  const auto& f = a.free_;
  for (size_t i = 0; i < f.size(); ++i) {
    if (f[i].first >= f[i].second) {
      *why = "empty or inverted range";
      return false;
    }
    if (i > 0 && f[i - 1].second >= f[i].first) {
      *why = "unsorted, overlapping or uncoalesced ranges";
      return false;
    }
  }
  std::vector<char> is_free(owner.size(), 0);
  for (const auto& r : f)
    for (int64_t g = r.first; g < r.second; ++g) {
      if (g < 0 || g >= (int64_t)owner.size()) {
        *why = "range outside the arena";
        return false;
      }
      is_free[g] = 1;
    }
  for (size_t g = 0; g < owner.size(); ++g)
    if ((owner[g] < 0) != (is_free[g] != 0)) {
      *why = "free list differs from the owned points";
      return false;
    }
  return true;
}

// lowest start of a free run of >= n points in the byte map, or -1
int64_t first_fit(const std::vector<int>& owner, int64_t n) {
  int64_t run = 0;
  for (int64_t g = 0; g < (int64_t)owner.size(); ++g) {
    run = owner[g] < 0 ? run + 1 : 0;
    if (run == n) return g - n + 1;
  }
  return -1;
}

bool one_case(std::mt19937_64& rng) {
  auto pick = [&](int64_t lo, int64_t hi) { return std::uniform_int_distribution<int64_t>(lo, hi)(rng); };
  const int64_t size = pick(1, 3000);
  pof::Arena a;
  a.init(size);
  std::vector<int> owner(size, -1);
  std::vector<std::pair<int64_t, int64_t>> live;  // (lo, n)
  const char* why = "";
  for (int op = 0; op < 400; ++op) {
    if (live.empty() || pick(0, 2) > 0) {
      const int64_t n = pick(0, 3) == 0 ? pick(1, size) : pick(1, 1 + size / 8);
      const int64_t want = first_fit(owner, n);
      const int64_t lo = a.alloc(n);
      if (lo != want) {
        fprintf(stderr, "FAIL alloc(%lld) = %lld, first fit %lld\n", (long long)n, (long long)lo, (long long)want);
        return false;
      }
      if (lo >= 0) {
        for (int64_t g = lo; g < lo + n; ++g) owner[g] = (int)live.size();
        live.push_back({lo, n});
      }
    } else {
      const size_t k = (size_t)pick(0, (int64_t)live.size() - 1);
      const auto r = live[k];
      a.release(r.first, r.second);
      for (int64_t g = r.first; g < r.first + r.second; ++g) owner[g] = -1;
      live[k] = live.back();
      live.pop_back();
      for (size_t j = 0; j < live.size(); ++j)  // renumber owners
        for (int64_t g = live[j].first; g < live[j].first + live[j].second; ++g) owner[g] = (int)j;
    }
    if (!check_free_list(a, owner, &why)) {
      fprintf(stderr, "FAIL after op %d: %s\n", op, why);
      return false;
    }
  }
  // release everything: one free range again
  for (const auto& r : live) a.release(r.first, r.second);
  if (a.free_.size() != 1 || a.free_[0].first != 0 || a.free_[0].second != size) {
    fprintf(stderr, "FAIL: arena not whole after releasing every range\n");
    return false;
  }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  const int cases = argc > 1 ? atoi(argv[1]) : 200;
  std::mt19937_64 rng(argc > 2 ? strtoull(argv[2], nullptr, 10) : 7);
  for (int i = 0; i < cases; ++i)
    if (!one_case(rng)) return 1;
  printf("ok %d\n", cases);
  return 0;
}
