// Plan of a batched IEKS solve: many independent problems of one state
// shape (D, d), each with its own number of steps, step size, field and
// parameters, solved by one pipeline of launches.  Host-only.
//
// Problem b owns the grid points [gb[b], gb[b] + ns[b]] of the concatenated
// trajectories and the steps [gb[b], gb[b] + ns[b]): step s maps grid point
// s to s + 1 (one index space for steps and grid points; the last index of
// each problem's range is a grid point with no step).  The chunked scan of
// the one-problem path is applied per problem: level-0 chunks and the groups
// of every level above never span two problems, and a problem's tree ends in
// a single element per problem at the top level, where its x0 (filter) and
// its terminal filtered state (smoother) are injected.  No arithmetic ever
// mixes two problems, so a problem's result depends only on its own data and
// on (C0, Cg, team sizes) -- not on which other problems share the batch.
//
// The workspace has a persistent part (indexed by problem id or global
// step: survives re-planning) and a level part (indexed by the plan's list
// of active problems: rebuilt when converged problems are dropped).
#pragma once

#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "pof_plan.h"

namespace pof {

constexpr int kBatchScalars = 16;  // doubles per problem (Scalar layout)

struct BatchShape {
  int D = 0, DY = 0, esz = 8;
  int C0 = 0;      // steps per level-0 chunk (0: rule)
  int Cg = 2;      // elements per group at levels >= 2
  int team = 0;    // lanes per team at level 0
  int team_up = 0; // lanes per team at levels >= 2
};

// Persistent part, fixed for the life of a batch.
struct BatchPersist {
  int64_t B = 0, n = 0, G = 0;  // problems, steps, grid points (the index space)
  size_t gb = 0;                // (B) int64 first grid point of each problem
  size_t ns = 0;                // (B) int64 steps of each problem
  size_t fld = 0;               // (B) int32 field id
  size_t p01 = 0;               // (B, 2) double Nordsieck scales
  size_t pscal = 0;             // (B, kBatchScalars) double
  size_t pscale = 0;            // (B) double sqrt(sigma^2) of the latest filter
  size_t frozen = 0;            // (B) int32
  size_t nactive = 0;           // int32 (+ pad)
  size_t H = 0, c = 0;          // (G, d, D), (G, d) indexed by step
  size_t selem = 0;             // smoother elements, SoA with stride G
  size_t means2 = 0;            // (G, D) second iterate buffer
  size_t host_tab = 0, host_tab_bytes = 0;  // gb | ns | fld | p01 (one upload)
  size_t total = 0;
};

// Level part, over the list of active problems.
struct BatchLevels {
  int64_t Ba = 0;          // active problems in this plan
  int64_t steps = 0;       // their steps
  int C0max = 0;           // longest chunk
  int nlev = 1;            // levels 1..nlev; cnt[nlev] == Ba
  int64_t cnt[kMaxLevels] = {0};
  size_t ap = 0, pc = 0;   // (Ba) int32 problem ids, (Ba + 1) int64 first chunk of each
  size_t cs = 0, ce = 0;   // (n1) int64 chunk step range [cs, ce)
  size_t cp = 0;           // (n1) int32 problem of each chunk
  size_t goff[kMaxLevels] = {0};  // l >= 2: (cnt[l] + 1) int64 group ranges into level l - 1
  size_t gp[kMaxLevels] = {0};    // l >= 2: (cnt[l]) int32 problem of each group
  size_t tab_bytes = 0;    // every table above, one upload from the start of the level part
  size_t felem[kMaxLevels] = {0}, fstate[kMaxLevels] = {0}, gelem[kMaxLevels] = {0}, gend[kMaxLevels] = {0};
  size_t partials = 0;     // (P_COUNT, n1) double
  size_t total = 0;
};

// Persistent part of a batch whose index space has G grid points (at least
// sum(n_steps) + B; more when problems sit in an arena with free space).
inline BatchPersist batch_persist(int64_t B, int64_t G, int D, int DY, int esz) {
  BatchPersist p;
  p.B = B;
  p.n = G - B;
  p.G = G;
  const int64_t NG = D + 2LL * D * D;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  // the host-built tables first, contiguous, so they go up in one copy
  p.host_tab = off;
  p.gb = take(sizeof(int64_t) * B);
  p.ns = take(sizeof(int64_t) * B);
  p.fld = take(sizeof(int32_t) * B);
  p.p01 = take(sizeof(double) * 2 * B);
  p.host_tab_bytes = off - p.host_tab;
  p.pscal = take(sizeof(double) * kBatchScalars * B);
  p.pscale = take(sizeof(double) * B);
  p.frozen = take(sizeof(int32_t) * B);
  p.nactive = take(16);
  p.H = take((size_t)esz * DY * D * G);
  p.c = take((size_t)esz * DY * G);
  p.selem = take((size_t)esz * NG * G);
  p.means2 = take((size_t)esz * D * G);
  p.total = off;
  return p;
}

// Chunk length rule when the caller gives none: about 8 x 8192 level-0
// chunks over the whole batch for 8-lane teams (several waves of the ~3600
// teams a GB300 holds at once, so the tail of the last wave is short),
// chunks as long as that allows, since the levels above level 0 cost more
// per step.  Measured on 512 FitzHugh-Nagumo problems (1.14 M steps): C0 =
// 32 (36 k chunks) 14.1 s, 64 (18 k) 14.9 s, 128 (9 k) 18.1 s.
inline int batch_pick_c0(int64_t total_steps, int lanes) {
  const int64_t target = 8 * (65536 / (lanes > 0 ? lanes : 1));
  int c = 4;
  while (c < 256 && total_steps / c > target) c *= 2;
  return c;
}

// Level tables of the plan over `active` (problem ids, in order); problem b
// has n_steps[b] steps from index gb[b], in chunks of c0[b] steps (sh.C0
// for every problem when c0 is null).  When `tab` is non-null it receives
// the tables' bytes (tab_bytes), laid out as in the workspace from the
// start of the level part.
inline BatchLevels batch_levels(const BatchShape& sh, const std::vector<int32_t>& active, const int64_t* n_steps,
                                const int64_t* gb, const int32_t* c0, std::vector<unsigned char>* tab) {
  BatchLevels L;
  const int64_t Ba = (int64_t)active.size();
  L.Ba = Ba;
  const int Cg = sh.Cg > 1 ? sh.Cg : 2;
  auto chunk = [&](int32_t b) -> int64_t { return c0 ? c0[b] : sh.C0; };
  // per-problem element counts per level
  std::vector<int64_t> cur(Ba);
  int64_t n1 = 0, steps = 0;
  int c0max = 1;
  for (int64_t k = 0; k < Ba; ++k) {
    const int64_t nb = n_steps[active[k]];
    const int64_t C = chunk(active[k]);
    cur[k] = (nb + C - 1) / C;
    n1 += cur[k];
    steps += nb;
    c0max = C > c0max ? (int)C : c0max;
  }
  L.steps = steps;
  L.C0max = c0max;
  L.cnt[1] = n1;
  int l = 1;
  std::vector<std::vector<int64_t>> per_level;  // counts per problem, per level
  per_level.push_back(cur);
  for (;;) {
    bool all_one = true;
    for (int64_t k = 0; k < Ba; ++k) all_one = all_one && cur[k] == 1;
    if (all_one || l + 1 >= kMaxLevels) break;
    int64_t tot = 0;
    for (int64_t k = 0; k < Ba; ++k) {
      cur[k] = (cur[k] + Cg - 1) / Cg;
      tot += cur[k];
    }
    ++l;
    L.cnt[l] = tot;
    per_level.push_back(cur);
  }
  L.nlev = l;
  const int D = sh.D;
  const int64_t NF = 3LL * D * D + 2 * D, NS = D + (int64_t)D * D, NG = D + 2LL * D * D;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  L.ap = take(sizeof(int32_t) * Ba);
  L.pc = take(sizeof(int64_t) * (Ba + 1));
  L.cs = take(sizeof(int64_t) * n1);
  L.ce = take(sizeof(int64_t) * n1);
  L.cp = take(sizeof(int32_t) * n1);
  for (int k = 2; k <= L.nlev; ++k) {
    L.goff[k] = take(sizeof(int64_t) * (L.cnt[k] + 1));
    L.gp[k] = take(sizeof(int32_t) * L.cnt[k]);
  }
  L.tab_bytes = off;
  for (int k = 1; k <= L.nlev; ++k) {
    L.felem[k] = take((size_t)sh.esz * NF * L.cnt[k]);
    L.fstate[k] = take((size_t)sh.esz * NS * L.cnt[k]);
    L.gelem[k] = take((size_t)sh.esz * NG * L.cnt[k]);
    L.gend[k] = take((size_t)sh.esz * NS * L.cnt[k]);
  }
  L.partials = take(sizeof(double) * 5 * n1);
  L.total = off;
  if (tab) {
    tab->assign(L.tab_bytes, 0);
    unsigned char* t = tab->data();
    int32_t* ap = reinterpret_cast<int32_t*>(t + L.ap);
    int64_t* pc = reinterpret_cast<int64_t*>(t + L.pc);
    int64_t* cs = reinterpret_cast<int64_t*>(t + L.cs);
    int64_t* ce = reinterpret_cast<int64_t*>(t + L.ce);
    int32_t* cp = reinterpret_cast<int32_t*>(t + L.cp);
    int64_t c = 0;
    for (int64_t k = 0; k < Ba; ++k) {
      const int32_t b = active[k];
      const int64_t C = chunk(b), s1 = gb[b] + n_steps[b];
      ap[k] = b;
      pc[k] = c;
      for (int64_t s = gb[b]; s < s1; s += C, ++c) {
        cs[c] = s;
        ce[c] = (s + C < s1) ? s + C : s1;
        cp[c] = b;
      }
    }
    pc[Ba] = c;
    for (int k = 2; k <= L.nlev; ++k) {
      int64_t* goff = reinterpret_cast<int64_t*>(t + L.goff[k]);
      int32_t* gp = reinterpret_cast<int32_t*>(t + L.gp[k]);
      const std::vector<int64_t>& below = per_level[k - 2];  // counts at level k - 1
      int64_t j = 0, base = 0;
      for (int64_t p = 0; p < Ba; ++p) {
        for (int64_t i = 0; i < below[p]; i += Cg, ++j) {
          goff[j] = base + i;
          gp[j] = active[p];
        }
        base += below[p];
      }
      goff[j] = base;
    }
  }
  return L;
}

}  // namespace pof
