// Property checks of libpof's host-side planners (pof_plan.h: one problem;
// pof_bplan.h: a batch), compiled with the host compiler alone and run by
// tests/test_plan_cpu.py.  Every kernel indexes the workspace through these
// offsets and tables, so each random case checks that
//   - the level counts follow the chunking (ceil divisions, the top rule),
//   - the workspace regions are 256-byte aligned, pairwise disjoint and
//     inside the reported total,
//   - the batch's level-0 chunks cover every problem's steps exactly once,
//     in order, never spanning two problems, and the groups of every level
//     above cover the level below exactly once, inside one problem, with at
//     most Cg members, ending in one element per problem.
// Prints "ok <cases>" and exits 0, or prints the first failure and exits 1.
#include <stdio.h>
#include <stdlib.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <utility>
#include <vector>

#include "pof_bplan.h"
#include "pof_plan.h"

namespace {

int g_fail = 0;
#define CHECK(cond, ...)                                  \
  do {                                                    \
    if (!(cond)) {                                        \
      fprintf(stderr, "FAIL %s:%d: %s | ", __FILE__, __LINE__, #cond); \
      fprintf(stderr, __VA_ARGS__);                       \
      fprintf(stderr, "\n");                              \
      g_fail = 1;                                         \
      return;                                             \
    }                                                     \
  } while (0)

struct Region {
  size_t off, bytes;
};

// regions: aligned, disjoint (empty ones ignored), inside total
bool regions_ok(std::vector<Region> r, size_t total, const char** why) {
  for (const Region& x : r) {
    if (x.off % 256) {
      *why = "unaligned";
      return false;
    }
    if (x.off + x.bytes > total) {
      *why = "past total";
      return false;
    }
  }
  r.erase(std::remove_if(r.begin(), r.end(), [](const Region& x) { return x.bytes == 0; }), r.end());
  std::sort(r.begin(), r.end(), [](const Region& a, const Region& b) { return a.off < b.off; });
  for (size_t i = 1; i < r.size(); ++i)
    if (r[i - 1].off + r[i - 1].bytes > r[i].off) {
      *why = "overlap";
      return false;
    }
  return true;
}

int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

void check_plan(std::mt19937_64& rng) {
  auto pick = [&](int64_t lo, int64_t hi) { return std::uniform_int_distribution<int64_t>(lo, hi)(rng); };
  int64_t n = pick(0, 3) == 0 ? pick(1, 64) : (int64_t)std::exp(std::uniform_real_distribution<double>(0, 21.5)(rng));
  if (n < 1) n = 1;
  const int D = (int)pick(2, 16), DY = (int)pick(1, 4), esz = pick(0, 1) ? 8 : 4;
  const bool solver = pick(0, 1), narrow = pick(0, 1);
  const int C0 = pick(0, 2) ? 0 : (int)pick(1, 64);
  const int Cg = pick(0, 2) ? 0 : (int)pick(2, 8);
  const int ks_max = pick(0, 2) == 0 ? 0 : (pick(0, 1) ? -1 : (int)pick(1, 5000));
  const pof::Plan p = pof::make_plan(n, D, DY, esz, solver, C0, Cg, narrow, ks_max);

  CHECK(p.C0 >= 1 && p.Cg >= 2, "C0 %d Cg %d", p.C0, p.Cg);
  if (C0 > 0) CHECK(p.C0 == C0, "C0 %d asked %d", p.C0, C0);
  if (C0 == 0) CHECK((p.C0 & (p.C0 - 1)) == 0 && p.C0 <= 64, "rule C0 %d", p.C0);
  CHECK(p.nlev >= 1 && p.nlev < pof::kMaxLevels, "nlev %d", p.nlev);
  CHECK(p.cnt[1] == cdiv(n, p.C0), "cnt1 %lld", (long long)p.cnt[1]);
  for (int l = 1; l < p.nlev; ++l)
    CHECK(p.cnt[l + 1] == cdiv(p.cnt[l], p.Cg) && p.cnt[l] > pof::kTop, "level %d", l);
  const int64_t top = p.cnt[p.nlev];
  if (!p.ks) CHECK(top <= pof::kTop, "tree top %lld", (long long)top);
  if (p.ks) {
    CHECK(top > pof::kTop, "ks top %lld", (long long)top);
    CHECK(top <= pof::ks_limit(D, ks_max) || p.nlev == pof::kMaxLevels - 1, "ks top %lld above limit",
          (long long)top);
  }
  const int64_t NF = 3LL * D * D + 2 * D, NS = D + (int64_t)D * D, NG = D + 2LL * D * D;
  std::vector<Region> r;
  for (int k = 1; k <= p.nlev; ++k) {
    r.push_back({p.felem[k], (size_t)(esz * NF * p.cnt[k])});
    r.push_back({p.fstate[k], (size_t)(esz * NS * p.cnt[k])});
    r.push_back({p.gelem[k], (size_t)(esz * NG * p.cnt[k])});
    r.push_back({p.gend[k], (size_t)(esz * NS * p.cnt[k])});
  }
  r.push_back({p.selem, (size_t)(esz * NG * n)});
  if (p.ks) r.push_back({p.ksbuf, (size_t)(esz * NF * top)});
  r.push_back({p.partials, sizeof(double) * 5 * (size_t)p.cnt[1]});
  r.push_back({p.scalars, sizeof(double) * 16});
  r.push_back({p.scale, (size_t)esz * 4});
  if (solver) {
    r.push_back({p.H, (size_t)(esz * DY * D * n)});
    r.push_back({p.c, (size_t)(esz * DY * n)});
    r.push_back({p.means2, (size_t)(esz * D * (n + 1))});
    r.push_back({p.params, (size_t)esz * 16});
  }
  const char* why = "";
  CHECK(regions_ok(r, p.total, &why), "plan regions: %s (n %lld D %d DY %d esz %d)", why, (long long)n, D, DY, esz);
}

void check_batch(std::mt19937_64& rng) {
  auto pick = [&](int64_t lo, int64_t hi) { return std::uniform_int_distribution<int64_t>(lo, hi)(rng); };
  const int64_t B = pick(1, 60);
  const int D = (int)pick(2, 12), DY = (int)pick(1, 3), esz = pick(0, 1) ? 8 : 4;
  // problems laid out in an index space with gaps (the serving arena)
  std::vector<int64_t> ns(B), gb(B);
  int64_t g = pick(0, 5);
  for (int64_t b = 0; b < B; ++b) {
    ns[b] = pick(0, 3) == 0 ? pick(1, 9) : pick(10, 6000);
    gb[b] = g;
    g += ns[b] + 1 + (pick(0, 3) == 0 ? pick(1, 40) : 0);
  }
  const int64_t G = g;
  pof::BatchShape sh;
  sh.D = D;
  sh.DY = DY;
  sh.esz = esz;
  sh.Cg = (int)pick(2, 6);
  sh.C0 = (int)(pick(0, 1) ? pof::batch_pick_c0(G - B, 8) : pick(1, 64));
  std::vector<int32_t> c0(B);
  const bool per_problem = pick(0, 1);
  for (int64_t b = 0; b < B; ++b) c0[b] = (int32_t)pick(1, 80);
  // active: a random subset, in increasing order
  std::vector<int32_t> active;
  for (int64_t b = 0; b < B; ++b)
    if (pick(0, 4)) active.push_back((int32_t)b);
  if (active.empty()) active.push_back((int32_t)pick(0, B - 1));

  const pof::BatchPersist P = pof::batch_persist(B, G, D, DY, esz);
  {
    const int64_t NG = D + 2LL * D * D;
    std::vector<Region> r = {{P.gb, 8 * (size_t)B},
                             {P.ns, 8 * (size_t)B},
                             {P.fld, 4 * (size_t)B},
                             {P.p01, 16 * (size_t)B},
                             {P.pscal, 8 * (size_t)pof::kBatchScalars * B},
                             {P.pscale, 8 * (size_t)B},
                             {P.frozen, 4 * (size_t)B},
                             {P.nactive, 16},
                             {P.H, (size_t)(esz * DY * D * G)},
                             {P.c, (size_t)(esz * DY * G)},
                             {P.selem, (size_t)(esz * NG * G)},
                             {P.means2, (size_t)(esz * D * G)}};
    const char* why = "";
    CHECK(regions_ok(r, P.total, &why), "persist regions: %s", why);
    CHECK(P.host_tab == 0 && P.host_tab_bytes >= P.p01 + 16 * (size_t)B && P.host_tab_bytes <= P.pscal,
          "host table span");
  }

  std::vector<unsigned char> tab;
  const int32_t* c0p = per_problem ? c0.data() : nullptr;
  const pof::BatchLevels L = pof::batch_levels(sh, active, ns.data(), gb.data(), c0p, &tab);
  const int64_t Ba = (int64_t)active.size();
  auto chunk_of = [&](int32_t b) -> int64_t { return per_problem ? c0[b] : sh.C0; };
  CHECK(L.Ba == Ba && tab.size() == L.tab_bytes, "Ba / table size");
  CHECK(L.cnt[L.nlev] == Ba, "top level holds %lld elements for %lld problems", (long long)L.cnt[L.nlev],
        (long long)Ba);
  int64_t steps = 0, n1 = 0;
  for (int32_t b : active) {
    steps += ns[b];
    n1 += cdiv(ns[b], chunk_of(b));
  }
  CHECK(L.steps == steps && L.cnt[1] == n1, "steps / chunks");

  const unsigned char* t = tab.data();
  const int32_t* ap = reinterpret_cast<const int32_t*>(t + L.ap);
  const int64_t* pc = reinterpret_cast<const int64_t*>(t + L.pc);
  const int64_t* cs = reinterpret_cast<const int64_t*>(t + L.cs);
  const int64_t* ce = reinterpret_cast<const int64_t*>(t + L.ce);
  const int32_t* cp = reinterpret_cast<const int32_t*>(t + L.cp);
  CHECK(pc[0] == 0 && pc[Ba] == n1, "chunk offsets ends");
  for (int64_t k = 0; k < Ba; ++k) {
    const int32_t b = active[k];
    CHECK(ap[k] == b, "active list");
    const int64_t C = chunk_of(b);
    int64_t s = gb[b];
    for (int64_t c = pc[k]; c < pc[k + 1]; ++c) {
      CHECK(cp[c] == b && cs[c] == s && ce[c] > cs[c] && ce[c] - cs[c] <= C, "chunk %lld of problem %d",
            (long long)c, b);
      s = ce[c];
    }
    CHECK(s == gb[b] + ns[b], "problem %d's chunks end at %lld, not %lld", b, (long long)s,
          (long long)(gb[b] + ns[b]));
  }
  // groups: level l >= 2 groups elements of level l - 1 of one problem
  std::vector<int32_t> owner(cp, cp + n1);  // problem of each element at the level below
  for (int l = 2; l <= L.nlev; ++l) {
    const int64_t* goff = reinterpret_cast<const int64_t*>(t + L.goff[l]);
    const int32_t* gp = reinterpret_cast<const int32_t*>(t + L.gp[l]);
    const int64_t below = L.cnt[l - 1];
    CHECK(goff[0] == 0 && goff[L.cnt[l]] == below, "level %d group ends", l);
    std::vector<int32_t> up(L.cnt[l]);
    for (int64_t j = 0; j < L.cnt[l]; ++j) {
      CHECK(goff[j + 1] > goff[j] && goff[j + 1] - goff[j] <= sh.Cg, "level %d group %lld size", l, (long long)j);
      for (int64_t i = goff[j]; i < goff[j + 1]; ++i)
        CHECK(owner[i] == gp[j], "level %d group %lld spans problems", l, (long long)j);
      up[j] = gp[j];
    }
    owner.swap(up);
  }
  for (int64_t k = 0; k < Ba; ++k) CHECK(owner[k] == active[k], "top element %lld", (long long)k);

  const int64_t NF = 3LL * D * D + 2 * D, NS = D + (int64_t)D * D, NG = D + 2LL * D * D;
  std::vector<Region> r = {{L.ap, 4 * (size_t)Ba}, {L.pc, 8 * (size_t)(Ba + 1)}, {L.cs, 8 * (size_t)n1},
                           {L.ce, 8 * (size_t)n1}, {L.cp, 4 * (size_t)n1}};
  for (int k = 2; k <= L.nlev; ++k) {
    r.push_back({L.goff[k], 8 * (size_t)(L.cnt[k] + 1)});
    r.push_back({L.gp[k], 4 * (size_t)L.cnt[k]});
  }
  for (const Region& x : r) CHECK(x.off + x.bytes <= L.tab_bytes, "table past tab_bytes");
  for (int k = 1; k <= L.nlev; ++k) {
    r.push_back({L.felem[k], (size_t)(esz * NF * L.cnt[k])});
    r.push_back({L.fstate[k], (size_t)(esz * NS * L.cnt[k])});
    r.push_back({L.gelem[k], (size_t)(esz * NG * L.cnt[k])});
    r.push_back({L.gend[k], (size_t)(esz * NS * L.cnt[k])});
  }
  r.push_back({L.partials, sizeof(double) * 5 * (size_t)n1});
  const char* why = "";
  CHECK(regions_ok(r, L.total, &why), "level regions: %s", why);
}

}  // namespace

int main(int argc, char** argv) {
  const int cases = argc > 1 ? atoi(argv[1]) : 2000;
  std::mt19937_64 rng(argc > 2 ? strtoull(argv[2], nullptr, 10) : 12345);
  for (int i = 0; i < cases && !g_fail; ++i) {
    check_plan(rng);
    if (!g_fail) check_batch(rng);
  }
  if (g_fail) return 1;
  printf("ok %d\n", cases);
  return 0;
}
