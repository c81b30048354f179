// Level structure and workspace layout of the chunked filter/smoother.
// Host-only; shared by the workspace-size queries and the launches so both
// always agree.
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>

namespace pof {

constexpr int kMaxLevels = 24;
constexpr int kTop = 2;  // at most this many elements are scanned by the single top team

struct Plan {
  int64_t n = 0;  // time steps
  int D = 0, DY = 0, esz = 8;
  int C0 = 4;  // steps per level-0 chunk
  int Cg = 8;  // elements per chunk at levels >= 1
  int nlev = 1;
  int team = 0;     // lanes per team of the level-0 team kernels (see l0_lanes)
  int team_up = 0;  // lanes per team at levels >= 1 and the tops
  // ks: the top level (cnt[nlev] > kTop elements) is scanned in parallel
  // (Kogge-Stone: ceil(log2 cnt[nlev]) steps of cnt[nlev] combines) instead
  // of by one team; ksbuf is its ping-pong partner (cnt[nlev] filter elements)
  bool ks = false;
  size_t ksbuf = 0;
  // means test of the convergence criterion: isclose(old, new, mrtol, matol)
  // (pof/convergence_criteria.py:10 uses rtol 1e-13 and numpy's atol 1e-8)
  double mrtol = 1e-13, matol = 1e-8;
  int64_t cnt[kMaxLevels] = {0};  // cnt[l], l = 1..nlev (cnt[nlev] <= kTop)
  size_t felem[kMaxLevels] = {0}, fstate[kMaxLevels] = {0}, gelem[kMaxLevels] = {0}, gend[kMaxLevels] = {0};
  size_t selem = 0, partials = 0, scalars = 0, scale = 0;
  size_t H = 0, c = 0, means2 = 0, params = 0;
  size_t total = 0;
};

// Lanes that work on one level-0 chunk: 1 (thread per chunk, state in
// registers) for small D, a team of 16 or 32 lanes (state in shared memory)
// from D = 6 on, where per-thread state would spill.  Must match
// Driver::kTeamL0 / TeamSize.
inline int team_lanes(int D, bool narrow) {
  const int wide = (2 * D <= 8) ? 8 : (2 * D <= 16 ? 16 : 32);
  return narrow ? (wide / 2 >= 4 ? wide / 2 : 4) : wide;
}
inline int l0_lanes(int D, bool narrow) { return D >= 6 ? team_lanes(D, narrow) : 1; }

// Level 0 is throughput-bound (narrow teams waste fewer lanes per FP64
// instruction); levels >= 1 are latency-bound (wide teams finish a combine
// sooner).  Measured on GB300: D = 8, narrow level 0 is 2x faster than wide.

inline int pick_c0(int64_t n, int lanes) {
  // Enough level-0 chunks to keep every SM sub-partition's FP64 pipe fed
  // (~16k lanes), chunks long enough that the per-step work (cheapest
  // formulas) dominates the general combines of the levels above.
  int c = lanes == 1 ? 4 : 2;
  const int64_t target = lanes == 1 ? 16384 : (65536 / lanes > 1024 ? 65536 / lanes : 1024);
  while (c < 64 && n / c > target) c *= 2;
  return c;
}

inline size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

// Nordsieck scales of the state's derivative orders 0 and 1 at step h:
// P = diag(|h|^(q-i+1/2) / (q-i)!), i = 0..q (pof/transitions.py:53-61);
// p0 = P[0, 0], p1 = P[1, 1].  Returns false unless D = d (q + 1), q >= 1.
inline bool nordsieck_scales(int D, int d, double h, double* p0, double* p1) {
  if (d < 1 || D % d) return false;
  const int q = D / d - 1;
  if (q < 1) return false;
  double f0 = 1.0, f1 = 1.0;
  for (int i = 2; i <= q; ++i) f0 *= i;
  for (int i = 2; i <= q - 1; ++i) f1 *= i;
  const double ah = fabs(h);
  *p0 = pow(ah, q + 0.5) / f0;
  *p1 = pow(ah, q - 0.5) / f1;
  return true;
}

// Largest top level scanned in parallel (Kogge-Stone) rather than by the
// tree: the levels of the binary tree with at most ~16k lanes of combines are
// latency-bound (a level costs one combine's latency on the way up and one
// on the way down), while a parallel-scan step costs one combine's latency
// and its extra work fits on the idle SMs -- 7 % less time per IEKS
// iteration on FHN q = 3, N = 2^16.  Off by default: on ill-conditioned
// problems its bracketing moves further from the reference's (logistic
// r = 3, q = 3, N = 300: 2e-5 against 7e-8 for the tree, after more IEKS
// iterations).  ks_max: 0 off, < 0 16384 / team lanes, else the limit.
inline int64_t ks_limit(int D, int ks_max) {
  if (ks_max >= 0) return ks_max;
  return 16384 / team_lanes(D, false);
}

// with_solver: also reserve the EK1 (H, c) buffers, a second means buffer
// and a parameter slot used by the IEKS loop.
inline Plan make_plan(int64_t n, int D, int DY, int esz, bool with_solver, int C0 = 0, int Cg = 0,
                      bool narrow = false, int ks_max = 0) {
  Plan p;
  p.n = n;
  p.D = D;
  p.DY = DY;
  p.esz = esz;
  p.team = team_lanes(D, !narrow);  // level 0: narrow unless told otherwise
  p.team_up = team_lanes(D, false);
  p.C0 = C0 > 0 ? C0 : pick_c0(n, l0_lanes(D, !narrow));
  // binary tree above level 0: the critical path holds one combine per level
  p.Cg = Cg > 1 ? Cg : 2;
  const int64_t NF = 3LL * D * D + 2 * D;  // filter element (A, b, U, eta, Z)
  const int64_t NS = D + (int64_t)D * D;   // state (m, L)
  const int64_t NG = D + 2LL * D * D;      // smoother element (g, E, Dm)
  p.cnt[1] = (n + p.C0 - 1) / p.C0;
  const int64_t ksk = ks_limit(D, ks_max);
  int l = 1;
  while (p.cnt[l] > kTop && p.cnt[l] > ksk && l + 1 < kMaxLevels) {
    p.cnt[l + 1] = (p.cnt[l] + p.Cg - 1) / p.Cg;
    ++l;
  }
  p.nlev = l;
  p.ks = p.cnt[l] > kTop;
  size_t off = 0;
  auto take = [&](int64_t elems) {
    size_t o = off;
    off = align_up(off + (size_t)elems * (size_t)esz);
    return o;
  };
  for (int k = 1; k <= p.nlev; ++k) {
    p.felem[k] = take(NF * p.cnt[k]);
    p.fstate[k] = take(NS * p.cnt[k]);
    p.gelem[k] = take(NG * p.cnt[k]);
    p.gend[k] = take(NS * p.cnt[k]);
  }
  p.selem = take(NG * n);
  if (p.ks) p.ksbuf = take(NF * p.cnt[p.nlev]);
  p.partials = off;
  off = align_up(off + sizeof(double) * 5 * (size_t)p.cnt[1]);
  p.scalars = off;
  off = align_up(off + sizeof(double) * 16);
  p.scale = take(4);
  if (with_solver) {
    p.H = take((int64_t)DY * D * n);
    p.c = take((int64_t)DY * n);
    p.means2 = take((int64_t)D * (n + 1));
    p.params = take(16);
  }
  p.total = off + 256;
  return p;
}

}  // namespace pof
