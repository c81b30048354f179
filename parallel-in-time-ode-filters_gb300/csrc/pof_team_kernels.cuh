// Levels >= 1 of the chunked scan with team-cooperative combines: one team
// of TS lanes per chunk (pof_team.cuh).  Same buffers and element order as
// the thread-per-chunk kernels of pof_kernels.cuh.
#pragma once

#include "pof_kernels.cuh"
#include "pof_team.cuh"

namespace pof {

template <int D>
struct TeamSize {
  static constexpr int v = (2 * D <= 8) ? 8 : (2 * D <= 16 ? 16 : 32);
};

template <typename WS, int TS>
struct TeamBlock {
  // teams per 64-thread block, fewer when the workspaces exceed ~40 KB
  static constexpr int per_warp_max = 64 / TS;
  static constexpr int fit = (int)(40960 / sizeof(WS));
  static constexpr int teams = fit < 1 ? 1 : (fit < per_warp_max ? fit : per_warp_max);
  static constexpr int threads = teams * TS;
};

// SoA element <-> team workspace slot
template <typename T, int TS, int D>
__device__ __forceinline__ void t_load_filt(const Team<TS>& tm, const T* base, int64_t n, int64_t e, T* A, T* b,
                                            T* U, T* eta, T* Z) {
  if (!POF_IN(e, n)) return;
  using FL = FiltLayout<D>;
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < FL::NF; f += TS) {
    const T v = base[f * n + e];
    if (f < FL::B)
      A[(f / D) * L1 + f % D] = v;
    else if (f < FL::U)
      b[f - FL::B] = v;
    else if (f < FL::ETA)
      U[((f - FL::U) / D) * L1 + (f - FL::U) % D] = v;
    else if (f < FL::Z)
      eta[f - FL::ETA] = v;
    else
      Z[((f - FL::Z) / D) * L1 + (f - FL::Z) % D] = v;
  }
}

template <typename T, int TS, int D>
__device__ __forceinline__ void t_store_filt(const Team<TS>& tm, T* base, int64_t n, int64_t e, const T* A,
                                             const T* b, const T* U, const T* eta, const T* Z) {
  if (!POF_IN(e, n)) return;
  using FL = FiltLayout<D>;
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < FL::NF; f += TS) {
    T v;
    if (f < FL::B)
      v = A[(f / D) * L1 + f % D];
    else if (f < FL::U)
      v = b[f - FL::B];
    else if (f < FL::ETA)
      v = U[((f - FL::U) / D) * L1 + (f - FL::U) % D];
    else if (f < FL::Z)
      v = eta[f - FL::ETA];
    else
      v = Z[((f - FL::Z) / D) * L1 + (f - FL::Z) % D];
    base[f * n + e] = v;
  }
}

// state (m, L) <-> slot
template <typename T, int TS, int D>
__device__ __forceinline__ void t_load_state(const Team<TS>& tm, const T* base, int64_t n, int64_t e, T* m, T* L) {
  if (!POF_IN(e, n)) return;
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < D + D * D; f += TS) {
    const T v = base[f * n + e];
    if (f < D)
      m[f] = v;
    else
      L[((f - D) / D) * L1 + (f - D) % D] = v;
  }
}
template <typename T, int TS, int D>
__device__ __forceinline__ void t_store_state(const Team<TS>& tm, T* base, int64_t n, int64_t e, const T* m,
                                              const T* L) {
  if (!POF_IN(e, n)) return;
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < D + D * D; f += TS) base[f * n + e] = (f < D) ? m[f] : L[((f - D) / D) * L1 + (f - D) % D];
}
template <typename T, int TS, int D>
__device__ __forceinline__ void t_load_state_plain(const Team<TS>& tm, const T* m0, const T* L0, T* m, T* L) {
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < D + D * D; f += TS) {
    if (f < D)
      m[f] = m0[f];
    else
      L[((f - D) / D) * L1 + (f - D) % D] = L0[f - D];
  }
}

// smoother element (g, E, Dm) <-> slot
template <typename T, int TS, int D>
__device__ __forceinline__ void t_load_smo(const Team<TS>& tm, const T* base, int64_t n, int64_t e, T* g, T* E,
                                           T* Dm) {
  if (!POF_IN(e, n)) return;
  using GL = SmoLayout<D>;
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < GL::NG; f += TS) {
    const T v = base[f * n + e];
    if (f < GL::E)
      g[f] = v;
    else if (f < GL::DM)
      E[((f - GL::E) / D) * L1 + (f - GL::E) % D] = v;
    else
      Dm[((f - GL::DM) / D) * L1 + (f - GL::DM) % D] = v;
  }
}
template <typename T, int TS, int D>
__device__ __forceinline__ void t_store_smo(const Team<TS>& tm, T* base, int64_t n, int64_t e, const T* g,
                                            const T* E, const T* Dm) {
  if (!POF_IN(e, n)) return;
  using GL = SmoLayout<D>;
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < GL::NG; f += TS) {
    T v;
    if (f < GL::E)
      v = g[f];
    else if (f < GL::DM)
      v = E[((f - GL::E) / D) * L1 + (f - GL::E) % D];
    else
      v = Dm[((f - GL::DM) / D) * L1 + (f - GL::DM) % D];
    base[f * n + e] = v;
  }
}

#define POF_TEAM_PROLOGUE(WS)                                             \
  using B_ = TeamBlock<WS, TS>;                                           \
  extern __shared__ __align__(16) unsigned char smem_raw_[];              \
  const int team_in_block = threadIdx.x / TS;                             \
  WS& w = reinterpret_cast<WS*>(smem_raw_)[team_in_block];               \
  const int64_t t = (int64_t)blockIdx.x * B_::teams + team_in_block;     \
  Team<TS> tm;

// Filter up-sweep at level l >= 1: fold C consecutive elements per team.
template <typename T, int D, int TS>
__global__ void k_filt_reduce_team(const T* __restrict__ in, int64_t nin, int C, T* __restrict__ out, int64_t nout) {
  using WS = FiltTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t >= nout) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < nin) ? i0 + C : nin;
  t_load_filt<T, TS, D>(tm, in, nin, i0, w.A1, w.b1, w.U1, w.e1, w.Z1);
  for (int64_t i = i0 + 1; i < i1; ++i) {
    t_load_filt<T, TS, D>(tm, in, nin, i, w.A2, w.b2, w.U2, w.e2, w.Z2);
    tm.sync();
    t_filt_combine<T, TS, D>(tm, w);
  }
  tm.sync();
  t_store_filt<T, TS, D>(tm, out, nout, t, w.A1, w.b1, w.U1, w.e1, w.Z1);
}

// state before element i+1 from the state before element i (element 0 of a
// level holds x0 and is absolute).
template <typename T, int D, int TS>
__device__ __forceinline__ void t_filt_advance(const Team<TS>& tm, FiltTeamWs<T, D>& w, const T* elems, int64_t n,
                                               int64_t i) {
  if (i == 0) {
    T* scratch = w.M;  // A, eta, Z of element 0 are not needed
    t_load_filt<T, TS, D>(tm, elems, n, 0, scratch, w.b1, w.U1, w.v1, scratch);
    tm.sync();
  } else {
    t_load_filt<T, TS, D>(tm, elems, n, i, w.A2, w.b2, w.U2, w.e2, w.Z2);
    tm.sync();
    t_filt_apply<T, TS, D>(tm, w);
  }
}

template <typename T, int D, int TS>
__global__ void k_filt_down_team(const T* __restrict__ elems, int64_t n, int C, const T* __restrict__ states_up,
                                 int64_t nup, T* __restrict__ states) {
  using WS = FiltTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t >= nup) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < n) ? i0 + C : n;
  t_load_state<T, TS, D>(tm, states_up, nup, t, w.b1, w.U1);
  tm.sync();
  for (int64_t i = i0; i < i1; ++i) {
    t_store_state<T, TS, D>(tm, states, n, i, w.b1, w.U1);
    tm.sync();
    if (i + 1 < i1) t_filt_advance<T, D, TS>(tm, w, elems, n, i);
  }
}

template <typename T, int D, int TS>
__global__ void k_filt_top_team(const T* __restrict__ elems, int64_t n, const T* __restrict__ x0m,
                                const T* __restrict__ x0L, T* __restrict__ states) {
  using WS = FiltTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t != 0) return;
  t_load_state_plain<T, TS, D>(tm, x0m, x0L, w.b1, w.U1);
  tm.sync();
  for (int64_t i = 0; i < n; ++i) {
    t_store_state<T, TS, D>(tm, states, n, i, w.b1, w.U1);
    tm.sync();
    if (i + 1 < n) t_filt_advance<T, D, TS>(tm, w, elems, n, i);
  }
}

// Smoother up-sweep at level l >= 1.
template <typename T, int D, int TS>
__global__ void k_smo_reduce_team(const T* __restrict__ in, int64_t nin, int C, T* __restrict__ out, int64_t nout) {
  using WS = SmoTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t >= nout) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < nin) ? i0 + C : nin;
  t_load_smo<T, TS, D>(tm, in, nin, i0, w.g2, w.E2, w.D2m);
  for (int64_t i = i0 + 1; i < i1; ++i) {
    t_load_smo<T, TS, D>(tm, in, nin, i, w.g1, w.E1, w.D1);
    tm.sync();
    t_smooth_combine<T, TS, D>(tm, w);
  }
  tm.sync();
  t_store_smo<T, TS, D>(tm, out, nout, t, w.g2, w.E2, w.D2m);
}

template <typename T, int D, int TS>
__global__ void k_smo_down_team(const T* __restrict__ elems, int64_t n, int C, const T* __restrict__ ends_up,
                                int64_t nup, T* __restrict__ ends) {
  using WS = SmoTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t >= nup) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < n) ? i0 + C : n;
  t_load_state<T, TS, D>(tm, ends_up, nup, t, w.g1, w.D1);
  tm.sync();
  for (int64_t i = i1 - 1; i >= i0; --i) {
    t_store_state<T, TS, D>(tm, ends, n, i, w.g1, w.D1);
    if (i > i0) {
      t_load_smo<T, TS, D>(tm, elems, n, i, w.g2, w.E2, w.D2m);
      tm.sync();
      t_smooth_apply<T, TS, D>(tm, w);
    }
    tm.sync();
  }
}

template <typename T, int D, int TS>
__global__ void k_smo_top_team(const T* __restrict__ elems, int64_t n, const T* __restrict__ mT,
                               const T* __restrict__ LT, T* __restrict__ ends) {
  using WS = SmoTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t != 0) return;
  t_load_state_plain<T, TS, D>(tm, mT, LT, w.g1, w.D1);
  tm.sync();
  for (int64_t i = n - 1; i >= 0; --i) {
    t_store_state<T, TS, D>(tm, ends, n, i, w.g1, w.D1);
    if (i > 0) {
      t_load_smo<T, TS, D>(tm, elems, n, i, w.g2, w.E2, w.D2m);
      tm.sync();
      t_smooth_apply<T, TS, D>(tm, w);
    }
    tm.sync();
  }
}

// ---------------------------------------------------------------------------
// Parallel scan of the top level (Kogge-Stone), one team per element.
// Element 0 of a level is absolute (it holds x0), so the prefix
// P_i = E_0 (x) ... (x) E_i carries the state after element i in its (b, U);
// step s computes P_i <- P_{i-s} (x) P_i for i >= s.  The last step writes
// the states before each element (states[0] = x0, states[i] = (b, U) of
// P_{i-1}) instead of the elements.  Same result as the binary tree up to
// rounding (another bracketing of the same associative operator,
// pof/parallel_filtsmooth/filter.py:117-142).
// ---------------------------------------------------------------------------
template <typename T, int D, int TS>
__global__ void k_filt_ks_team(const T* __restrict__ in, int64_t K, int64_t s, int last, T* __restrict__ out,
                               T* __restrict__ states, const T* __restrict__ x0m, const T* __restrict__ x0L) {
  using WS = FiltTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t >= K || (last && t + 1 >= K && t != 0)) return;  // P_{K-1} is not needed
  if (t >= s) {
    t_load_filt<T, TS, D>(tm, in, K, t - s, w.A1, w.b1, w.U1, w.e1, w.Z1);
    t_load_filt<T, TS, D>(tm, in, K, t, w.A2, w.b2, w.U2, w.e2, w.Z2);
    tm.sync();
    t_filt_combine<T, TS, D>(tm, w);
  } else {
    t_load_filt<T, TS, D>(tm, in, K, t, w.A1, w.b1, w.U1, w.e1, w.Z1);
  }
  tm.sync();
  if (!last) {
    t_store_filt<T, TS, D>(tm, out, K, t, w.A1, w.b1, w.U1, w.e1, w.Z1);
    return;
  }
  if (t + 1 < K) t_store_state<T, TS, D>(tm, states, K, t + 1, w.b1, w.U1);
  if (t == 0) {
    t_load_state_plain<T, TS, D>(tm, x0m, x0L, w.b2, w.U2);
    tm.sync();
    t_store_state<T, TS, D>(tm, states, K, 0, w.b2, w.U2);
  }
}

// The last element of the smoother's top level made absolute: the terminal
// state (mT, LT) pushed through it, stored as (g = m, E = 0, Dm = L).
template <typename T, int D, int TS>
__global__ void k_smo_abs_team(T* __restrict__ elems, int64_t K, const T* __restrict__ mT,
                               const T* __restrict__ LT) {
  using WS = SmoTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t != 0) return;
  t_load_state_plain<T, TS, D>(tm, mT, LT, w.g1, w.D1);
  t_load_smo<T, TS, D>(tm, elems, K, K - 1, w.g2, w.E2, w.D2m);
  tm.sync();
  t_smooth_apply<T, TS, D>(tm, w);
  t_fill<T, TS, D, D, Ld<D>::v>(tm, w.E2, T(0), T(0));
  tm.sync();
  t_store_smo<T, TS, D>(tm, elems, K, K - 1, w.g1, w.E2, w.D1);
}

// Suffix scan of the smoother's top level after k_smo_abs_team: S_i <- S_i o
// S_{i+s} for i + s < K (pof/parallel_filtsmooth/smoother.py:53-63); S_i is
// absolute and its (g, Dm) is the state at the start of block i.  The last
// step writes ends[i - 1] = (g, Dm) of S_i and ends[K - 1] = (mT, LT).
template <typename T, int D, int TS>
__global__ void k_smo_ks_team(const T* __restrict__ in, int64_t K, int64_t s, int last, T* __restrict__ out,
                              T* __restrict__ ends, const T* __restrict__ mT, const T* __restrict__ LT) {
  using WS = SmoTeamWs<T, D>;
  POF_TEAM_PROLOGUE(WS)
  if (t >= K || (last && t == 0 && K > 1)) return;  // S_0 is not needed
  if (t + s < K) {
    t_load_smo<T, TS, D>(tm, in, K, t, w.g2, w.E2, w.D2m);
    t_load_smo<T, TS, D>(tm, in, K, t + s, w.g1, w.E1, w.D1);
    tm.sync();
    t_smooth_combine<T, TS, D>(tm, w);
  } else {
    t_load_smo<T, TS, D>(tm, in, K, t, w.g2, w.E2, w.D2m);
  }
  tm.sync();
  if (!last) {
    t_store_smo<T, TS, D>(tm, out, K, t, w.g2, w.E2, w.D2m);
    return;
  }
  t_store_state<T, TS, D>(tm, ends, K, t - 1, w.g2, w.D2m);
  if (t == K - 1) {
    t_load_state_plain<T, TS, D>(tm, mT, LT, w.g1, w.D1);
    tm.sync();
    t_store_state<T, TS, D>(tm, ends, K, K - 1, w.g1, w.D1);
  }
}

// ---------------------------------------------------------------------------
// Level 0 with teams (large D, where per-thread state does not fit registers)
// ---------------------------------------------------------------------------

// Transition model of a level-0 kernel and QL^{-1} (objective terms): one
// copy per block, shared by its teams, when it is the same for every step
// (PS = false: the preconditioned IWP); one per team, reloaded each step,
// when it varies (PS = true).
template <typename T, int D>
struct FQ {
  T F[D * Ld<D>::v], QL[D * Ld<D>::v], QLi[D * Ld<D>::v];
  int wq;  // D when QL is lower-triangular (t_tria's wlow for [F L, QL]), else 0
  int wf;  // Q when F is block-diagonal with upper-triangular Q x Q blocks, else 0
};

// 1 if the (D x D, row-major, leading dimension ld) entry (i, k) of F breaks
// the block-upper-triangular pattern with blocks of Q (Q = 0: no pattern)
template <typename T>
__device__ __forceinline__ bool breaks_fblocks(T v, int i, int k, int Q) {
  return Q <= 0 || (v != T(0) && (k < i || k >= (i / Q + 1) * Q));
}

template <typename Base, typename T, int D, bool PS>
struct WithFQ : Base {};
template <typename Base, typename T, int D>
struct WithFQ<Base, T, D, true> : Base {
  FQ<T, D> fq;
};

template <typename T, int D, int DY>
struct L0KFBase {
  StepKFWs<T, D, DY> s;
  T mold[D], r[D];
};
template <typename T, int D, int DY>
struct L0FoldBase {
  StepFoldWs<T, D, DY> s;
};
template <typename T, int D>
struct SmoL0Base {
  SmoTeamWs<T, D> s;
  T mnext[D], r[D];
};
template <typename T, int D, int DY, bool PS>
using L0KFWs = WithFQ<L0KFBase<T, D, DY>, T, D, PS>;
template <typename T, int D, int DY, bool PS>
using L0FoldWs = WithFQ<L0FoldBase<T, D, DY>, T, D, PS>;
template <typename T, int D, bool PS>
using SmoL0Ws = WithFQ<SmoL0Base<T, D>, T, D, PS>;

// Bytes of the block-shared transition model in front of the team array.
template <typename T, int D, bool PS>
struct FQHeader {
  static constexpr int bytes = PS ? 0 : (int)sizeof(FQ<T, D>);
};

// teams per block of a level-0 kernel with a shared header of HB bytes:
// up to 64 / TS teams within the default 48 KB of dynamic shared memory.
// Team workspaces are `stride` bytes apart, stride = 64 (mod 128): the two
// 8-lane teams of a half-warp then sit 8 doubles apart in the 32 banks, so a
// column of an odd-leading-dimension matrix read one row per lane (and a row
// read one column per lane) by both teams at once hits 32 distinct banks.
template <typename WS, int TS, int HB>
struct TeamBlockH {
  static constexpr int stride = (int)(((sizeof(WS) + 63) / 128) * 128 + 64);
  static constexpr int per_warp_max = 64 / TS;
  static constexpr int fit = (int)((49152 - HB) / stride);
  static constexpr int teams = fit < 1 ? 1 : (fit < per_warp_max ? fit : per_warp_max);
  static constexpr int threads = teams * TS;
  static constexpr int smem = HB + teams * stride;
};

template <typename T, int TS, int D>
__device__ __forceinline__ void t_load_FQ(const Team<TS>& tm, FQ<T, D>& q, const StepModel& sm, int64_t s, int Q) {
  constexpr int L1 = Ld<D>::v;
  const T* F = static_cast<const T*>(sm.F) + s * sm.ft_stride;
  const T* QL = static_cast<const T*>(sm.QL) + s * sm.ft_stride;
  bool upper = false, fdense = false;
  for (int f = tm.r; f < D * D; f += TS) {
    q.F[(f / D) * L1 + f % D] = F[f];
    q.QL[(f / D) * L1 + f % D] = QL[f];
    upper |= (f % D > f / D) && QL[f] != T(0);
    fdense |= breaks_fblocks(F[f], f / D, f % D, Q);
  }
  const bool any_upper = __any_sync(tm.mask, upper);
  const bool any_fdense = __any_sync(tm.mask, fdense);
  if (tm.r == 0) {
    q.wq = any_upper ? 0 : D;
    q.wf = any_fdense ? 0 : Q;
  }
}

// QL^{-1} by forward substitution on the identity (objective terms)
template <typename T, int TS, int D>
__device__ __forceinline__ void t_inv_lower(const Team<TS>& tm, const T* QL, T* QLi) {
  constexpr int L1 = Ld<D>::v;
  t_fill<T, TS, D, D, L1>(tm, QLi, T(0), T(1));
  tm.sync();
  t_trsm_l<T, TS, D, D, L1, L1>(tm, QL, QLi);
  tm.sync();
}

// The block's shared transition model (every thread of the block takes
// part: call before any team leaves).
template <typename T, int TS, int D>
__device__ __forceinline__ void load_fq_block(const Team<TS>& tm, FQ<T, D>& q, const T* F, const T* QL, int Q) {
  constexpr int L1 = Ld<D>::v;
  int upper = 0, fdense = 0;
  for (int f = threadIdx.x; f < D * D; f += blockDim.x) {
    q.F[(f / D) * L1 + f % D] = F[f];
    q.QL[(f / D) * L1 + f % D] = QL[f];
    upper |= (f % D > f / D) && QL[f] != T(0);
    fdense |= breaks_fblocks(F[f], f / D, f % D, Q);
  }
  upper = __syncthreads_or(upper);
  fdense = __syncthreads_or(fdense);
  if (threadIdx.x == 0) {
    q.wq = upper ? 0 : D;
    q.wf = fdense ? 0 : Q;
  }
  if (threadIdx.x < TS) t_inv_lower<T, TS, D>(tm, q.QL, q.QLi);
  __syncthreads();
}

// || QL^{-1} (a - F b) ||^2 with QLi = QL^{-1}; every lane gets the value.
template <typename T, int TS, int D>
__device__ __forceinline__ T t_objective(const Team<TS>& tm, const T* F, const T* QLi, const T* a, const T* b,
                                         T* r) {
  constexpr int L1 = Ld<D>::v;
  for (int i = tm.r; i < D; i += TS) {
    T s = a[i];
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(-F[i * L1 + k], b[k], s);
    r[i] = s;
  }
  tm.sync();
  T part = T(0);
  for (int i = tm.r; i < D; i += TS) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(QLi[i * L1 + k], r[k], s);
    part = fma(s, s, part);
  }
  const T tot = tm.sum(part);
  tm.sync();
  return tot;
}

// Prologue of a level-0 kernel: the shared header (when PS is false), this
// thread's team workspace ws_, its chunk t and the team handle; `fq` is the
// transition model the team reads (the block's, or its own copy).
#define POF_L0_PROLOGUE(WS, PS)                                                          \
  constexpr int HB_ = FQHeader<T, D, PS>::bytes;                                         \
  using B_ = TeamBlockH<WS, TS, HB_>;                                                    \
  extern __shared__ __align__(16) unsigned char smem_raw_[];                             \
  const int team_in_block = threadIdx.x / TS;                                            \
  WS& ws_ = *reinterpret_cast<WS*>(smem_raw_ + HB_ + team_in_block * B_::stride);     \
  const int64_t t = (int64_t)blockIdx.x * B_::teams + team_in_block;                    \
  Team<TS> tm;                                                                           \
  FQ<T, D>& fq = fq_ref<PS, T, D>(ws_, smem_raw_);

template <bool PS, typename T, int D, typename WS>
__device__ __forceinline__ FQ<T, D>& fq_ref(WS& ws, unsigned char* smem) {
  if constexpr (PS)
    return ws.fq;
  else
    return *reinterpret_cast<FQ<T, D>*>(smem);
}

// Per-step transition model into the team's copy (PS), or nothing.
template <bool PS, typename T, int TS, int D>
__device__ __forceinline__ void fq_step(const Team<TS>& tm, FQ<T, D>& q, const StepModel& sm, int64_t s,
                                        bool objective, int Q) {
  if constexpr (PS) {
    tm.sync();
    t_load_FQ<T, TS, D>(tm, q, sm, s, Q);
    tm.sync();
    if (objective) t_inv_lower<T, TS, D>(tm, q.QL, q.QLi);
  }
}

template <typename T, int D, int DY, int TS, bool PS>
__global__ void k_filt_l0_reduce_team(int64_t n, int C0, StepModel sm, const T* __restrict__ x0m,
                                      const T* __restrict__ x0L, T* __restrict__ out, int64_t n1) {
  using WS = L0FoldWs<T, D, DY, PS>;
  POF_L0_PROLOGUE(WS, PS)
  if constexpr (!PS)
    load_fq_block<T, TS, D>(tm, fq, static_cast<const T*>(sm.F), static_cast<const T*>(sm.QL), D / DY);
  if (t >= n1) return;
  StepFoldWs<T, D, DY>& w = ws_.s;
  constexpr int L1 = Ld<D>::v;
  const int64_t s0 = t * C0;
  const int64_t s1 = (s0 + C0 < n) ? s0 + C0 : n;
  if (t == 0) {
    t_load_state_plain<T, TS, D>(tm, x0m, x0L, w.m, w.L);
    for (int64_t s = s0; s < s1; ++s) {
      if (!POF_IN(s, n)) break;
      fq_step<PS, T, TS, D>(tm, fq, sm, s, false, D / DY);
      StepView<T, D, DY> v(sm, s);
      t_load_step<T, TS, D, DY>(tm, w, v.H, v.c, v.R);
      tm.sync();
      t_kf_step<T, TS, D, DY, false>(tm, w, fq.F, fq.QL, StepStruct{fq.wq, fq.wf, sm.R == nullptr});
    }
    t_fill<T, TS, D, D, L1>(tm, w.A, T(0), T(0));
    t_fill<T, TS, D, D, L1>(tm, w.Z, T(0), T(0));
    for (int i = tm.r; i < D; i += TS) w.eta[i] = T(0);
    tm.sync();
    t_store_filt<T, TS, D>(tm, out, n1, t, w.A, w.m, w.L, w.eta, w.Z);
  } else {
    t_fill<T, TS, D, D, L1>(tm, w.A, T(0), T(1));
    t_fill<T, TS, D, D, L1>(tm, w.L, T(0), T(0));
    t_fill<T, TS, D, D, L1>(tm, w.Z, T(0), T(0));
    for (int i = tm.r; i < D; i += TS) {
      w.b[i] = T(0);
      w.eta[i] = T(0);
    }
    for (int64_t s = s0; s < s1; ++s) {
      if (!POF_IN(s, n)) break;
      fq_step<PS, T, TS, D>(tm, fq, sm, s, false, D / DY);
      StepView<T, D, DY> v(sm, s);
      t_load_step<T, TS, D, DY>(tm, w, v.H, v.c, v.R);
      tm.sync();
      t_cond_fold_step<T, TS, D, DY>(tm, w, fq.F, fq.QL, StepStruct{fq.wq, fq.wf, sm.R == nullptr});
    }
    tm.sync();
    t_store_filt<T, TS, D>(tm, out, n1, t, w.A, w.b, w.L, w.eta, w.Z);
  }
}

template <typename T, int D, int DY, int TS, bool PS>
__global__ void k_filt_l0_down_team(int64_t n, int C0, StepModel sm, const T* __restrict__ states1, int64_t n1,
                                    T* __restrict__ means, T* __restrict__ chols, T* __restrict__ selems,
                                    double* __restrict__ partials) {
  using WS = L0KFWs<T, D, DY, PS>;
  POF_L0_PROLOGUE(WS, PS)
  if constexpr (!PS)
    load_fq_block<T, TS, D>(tm, fq, static_cast<const T*>(sm.F), static_cast<const T*>(sm.QL), D / DY);
  if (t >= n1) return;
  StepKFWs<T, D, DY>& w = ws_.s;
  using GL = SmoLayout<D>;
  constexpr int L1 = Ld<D>::v, L2 = Ld<2 * D>::v;
  const int64_t s0 = t * C0;
  const int64_t s1 = (s0 + C0 < n) ? s0 + C0 : n;
  t_load_state<T, TS, D>(tm, states1, n1, t, w.m, w.L);
  tm.sync();
  if (t == 0) {
    for (int f = tm.r; f < D + D * D; f += TS) {
      if (f < D)
        means[f] = w.m[f];
      else
        chols[f - D] = w.L[((f - D) / D) * L1 + (f - D) % D];
    }
  }
  double ssq = 0.0, nll = 0.0, fobj = 0.0;
  for (int64_t s = s0; s < s1; ++s) {
    if (!POF_IN(s, n)) break;
    fq_step<PS, T, TS, D>(tm, fq, sm, s, true, D / DY);
    StepView<T, D, DY> v(sm, s);
    t_load_step<T, TS, D, DY>(tm, w, v.H, v.c, v.R);
    for (int i = tm.r; i < D; i += TS) ws_.mold[i] = w.m[i];
    tm.sync();
    t_kf_step<T, TS, D, DY, true>(tm, w, fq.F, fq.QL, StepStruct{fq.wq, fq.wf, sm.R == nullptr});
    ssq += (double)w.sc[0];
    nll += (double)w.sc[1];
    fobj += (double)t_objective<T, TS, D>(tm, fq.F, fq.QLi, ws_.mold, w.m, ws_.r);
    // smoother element of grid s: g, E (stored transposed in w.E), Dm = Y[:, D:]
    for (int f = tm.r; f < GL::NG; f += TS) {
      T val;
      if (f < GL::E)
        val = w.g[f];
      else if (f < GL::DM)
        val = w.E[((f - GL::E) % D) * L1 + (f - GL::E) / D];
      else
        val = w.Y[((f - GL::DM) / D) * L2 + D + (f - GL::DM) % D];
      selems[f * n + s] = val;
    }
    for (int f = tm.r; f < D + D * D; f += TS) {
      if (f < D)
        means[(s + 1) * D + f] = w.m[f];
      else
        chols[(s + 1) * D * D + f - D] = w.L[((f - D) / D) * L1 + (f - D) % D];
    }
    tm.sync();
  }
  if (tm.r == 0) {
    partials[P_SSQ * n1 + t] = ssq;
    partials[P_NLL * n1 + t] = nll;
    partials[P_FOBJ * n1 + t] = fobj;
  }
}

template <typename T, int D, int TS, bool PS>
__global__ void k_smo_l0_down_team(int64_t n, int C0, const T* __restrict__ F, const T* __restrict__ QL,
                                   int64_t ft_stride, const T* __restrict__ selems, const T* __restrict__ ends1,
                                   int64_t n1, T* __restrict__ means, T* __restrict__ chols,
                                   const T* __restrict__ scale, const T* __restrict__ means_old, double c_mrtol,
                                   double c_matol, double* __restrict__ partials) {
  using WS = SmoL0Ws<T, D, PS>;
  POF_L0_PROLOGUE(WS, PS)
  if constexpr (!PS) load_fq_block<T, TS, D>(tm, fq, F, QL, 0);
  if (t >= n1) return;
  SmoTeamWs<T, D>& w = ws_.s;
  constexpr int L1 = Ld<D>::v;
  const int64_t s0 = t * C0;
  const int64_t s1 = (s0 + C0 < n) ? s0 + C0 : n;
  const T sc = scale ? *scale : T(1);
  const StepModel sm{F, QL, ft_stride, nullptr, nullptr, nullptr, 0};
  t_load_state<T, TS, D>(tm, ends1, n1, t, w.g1, w.D1);
  tm.sync();
  double sobj = 0.0, notclose = 0.0;
  auto close_count = [&](int64_t k) {
    if (!means_old) return;
    for (int i = tm.r; i < D; i += TS) {
      const double a = (double)means_old[k * D + i], b = (double)w.g1[i];
      bool ok;
      if (isfinite(a) && isfinite(b))
        ok = fabs(a - b) <= c_matol + c_mrtol * fabs(b);
      else
        ok = (a == b);
      notclose += ok ? 0.0 : 1.0;
    }
  };
  if (s1 == n) {
    close_count(n);
    if (scale)
      for (int f = tm.r; f < D * D; f += TS) chols[n * D * D + f] = w.D1[(f / D) * L1 + f % D] * sc;
  }
  for (int64_t k = s1 - 1; k >= s0; --k) {
    if (!POF_IN(k, n)) break;
    fq_step<PS, T, TS, D>(tm, fq, sm, k, true, 0);
    for (int i = tm.r; i < D; i += TS) ws_.mnext[i] = w.g1[i];
    t_load_smo<T, TS, D>(tm, selems, n, k, w.g2, w.E2, w.D2m);
    tm.sync();
    t_smooth_apply<T, TS, D>(tm, w);
    sobj += (double)t_objective<T, TS, D>(tm, fq.F, fq.QLi, w.g1, ws_.mnext, ws_.r);
    close_count(k);
    for (int f = tm.r; f < D + D * D; f += TS) {
      if (f < D)
        means[k * D + f] = w.g1[f];
      else
        chols[k * D * D + f - D] = w.D1[((f - D) / D) * L1 + (f - D) % D] * sc;
    }
    tm.sync();
  }
  notclose = (double)tm.sum(notclose);
  if (tm.r == 0) {
    partials[P_SOBJ * n1 + t] = sobj;
    partials[P_NOTCLOSE * n1 + t] = notclose;
  }
}

#undef POF_L0_PROLOGUE

#undef POF_TEAM_PROLOGUE

}  // namespace pof
