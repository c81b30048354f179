// Batched IEKS kernels: the chunked scan of the one-problem path, segmented
// per problem (layout and invariants in pof_bplan.h).  Team-cooperative
// everywhere (pof_team.cuh): one team of TS lanes per level-0 chunk or per
// group of a level above.  Teams of problems that have converged (frozen)
// return at once, so their outputs stay as they were when they converged.
#pragma once

#include "pof_bplan.h"
#include "pof_driver.cuh"

namespace pof {

// Device view of the tables of a plan (persistent + level part).
struct BView {
  const int64_t* gb;      // (B) first grid point of each problem (= index of its first step)
  const int64_t* ns;      // (B) steps of each problem
  const int32_t* fld;     // (B)
  const double* p01;      // (B, 2)
  const int32_t* frozen;  // (B)
  const int32_t* ap;      // (Ba)
  const int64_t* pc;      // (Ba + 1)
  const int64_t* cs;      // (n1)
  const int64_t* ce;      // (n1)
  const int32_t* cp;      // (n1)
  const double* rtol;     // (B) objective rtol of crit per problem, or null (a shared value)
  const int64_t* maxit;   // (B) maxiters per problem, or null (a shared value)
  const volatile int32_t* cancel;  // (B) host-set cancel flags (mapped host memory), or null
  int64_t n;              // grid points of the index space (SoA stride of the smoother elements)
  int64_t nb;             // problem slots of the index space (bound of every problem index)
  int64_t n1;             // level-0 chunks
  int64_t Ba;             // problems of the plan
  int C0;                 // longest chunk
};

#define POF_BTEAM_PROLOGUE(WS)                                            \
  using B_ = TeamBlock<WS, TS>;                                           \
  extern __shared__ __align__(16) unsigned char smem_raw_[];              \
  const int team_in_block = threadIdx.x / TS;                             \
  WS& ws_ = reinterpret_cast<WS*>(smem_raw_)[team_in_block];             \
  const int64_t t = (int64_t)blockIdx.x * B_::teams + team_in_block;     \
  Team<TS> tm;

// Level-0 batch kernels: the block shares one copy of F, QL, QL^{-1} (the
// preconditioned transition model is the same for every step and problem);
// Q: block size of F's block-upper-triangular pattern to test for (0: none).
#define POF_BL0_PROLOGUE(WS, Q)                                                          \
  constexpr int HB_ = FQHeader<T, D, false>::bytes;                                      \
  using B_ = TeamBlockH<WS, TS, HB_>;                                                    \
  extern __shared__ __align__(16) unsigned char smem_raw_[];                             \
  const int team_in_block = threadIdx.x / TS;                                            \
  WS& ws_ = *reinterpret_cast<WS*>(smem_raw_ + HB_ + team_in_block * B_::stride);     \
  const int64_t t = (int64_t)blockIdx.x * B_::teams + team_in_block;                    \
  Team<TS> tm;                                                                           \
  FQ<T, D>& fq = *reinterpret_cast<FQ<T, D>*>(smem_raw_);                               \
  load_fq_block<T, TS, D>(tm, fq, F, QL, Q);

// EK1 linearization (pof/step.py:12-22, observations.py:35-40) at the
// previous iterate, one thread per step of an active chunk: the residual
// E1 x - f(E0 x) of the step's problem (own field, parameters and Nordsieck
// scales p0, p1).  Same arithmetic as k_linearize.
template <typename T, int D, int DY>
__global__ void kb_linearize(BView v, const T* __restrict__ params, const T* __restrict__ means, T* __restrict__ H,
                             T* __restrict__ c) {
  constexpr int Q1 = D / DY;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t t = i / v.C0;
  if (t >= v.n1) return;
  const int b = v.cp[t];
  if (!POF_IN(b, v.nb) || v.frozen[b]) return;
  const int64_t s = v.cs[t] + i % v.C0;
  if (s >= v.ce[t] || !POF_IN(s + 1, v.n)) return;
  const T p0 = (T)v.p01[2 * b], p1 = (T)v.p01[2 * b + 1];
  const T* m = means + (s + 1) * D;
  T y[DY], f[DY], J[DY * DY];
#pragma unroll
  for (int k = 0; k < DY; ++k) y[k] = p0 * m[k * Q1];
  field_eval<T, DY>(v.fld[b], params + 4 * b, y, f, J);
  T h[DY * D];
#pragma unroll
  for (int r = 0; r < DY; ++r) {
#pragma unroll
    for (int k = 0; k < D; ++k) h[r * D + k] = T(0);
#pragma unroll
    for (int j = 0; j < DY; ++j) h[r * D + j * Q1] = -(J[r * DY + j] * p0);
    h[r * D + r * Q1 + 1] += p1;
  }
#pragma unroll
  for (int r = 0; r < DY; ++r) {
    T res = p1 * m[r * Q1 + 1] - f[r];
    T hm = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) hm = fma(h[r * D + k], m[k], hm);
    c[s * DY + r] = res - hm;
  }
#pragma unroll
  for (int k = 0; k < DY * D; ++k) H[s * DY * D + k] = h[k];
}

// Filter level 0: conditional fold of every chunk (the chunk's element of
// the filtering scan, filter.py:57-94 composed over its steps).
template <typename T, int D, int DY, int TS>
__global__ void kb_filt_l0_reduce(BView v, const T* __restrict__ F, const T* __restrict__ QL,
                                  const T* __restrict__ H, const T* __restrict__ c, T* __restrict__ out) {
  using WS = L0FoldWs<T, D, DY, false>;
  POF_BL0_PROLOGUE(WS, D / DY)
  if (t >= v.n1) return;
  if (v.frozen[v.cp[t]]) return;
  StepFoldWs<T, D, DY>& w = ws_.s;
  constexpr int L1 = Ld<D>::v;
  const int64_t s0 = v.cs[t], s1 = v.ce[t];
  t_fill<T, TS, D, D, L1>(tm, w.A, T(0), T(1));
  t_fill<T, TS, D, D, L1>(tm, w.L, T(0), T(0));
  t_fill<T, TS, D, D, L1>(tm, w.Z, T(0), T(0));
  for (int i = tm.r; i < D; i += TS) {
    w.b[i] = T(0);
    w.eta[i] = T(0);
  }
  for (int64_t s = s0; s < s1; ++s) {
    if (!POF_IN(s, v.n)) break;
    t_load_step<T, TS, D, DY>(tm, w, H + s * DY * D, c + s * DY, nullptr);
    tm.sync();
    t_cond_fold_step<T, TS, D, DY>(tm, w, fq.F, fq.QL, StepStruct{fq.wq, fq.wf, true});
  }
  tm.sync();
  t_store_filt<T, TS, D>(tm, out, v.n1, t, w.A, w.b, w.L, w.eta, w.Z);
}

// Filter levels >= 2: fold each group [goff[j], goff[j+1]) of level l - 1.
template <typename T, int D, int TS>
__global__ void kb_filt_reduce(const int64_t* __restrict__ goff, const int32_t* __restrict__ gp,
                               const int32_t* __restrict__ frozen, const T* __restrict__ in, int64_t nin,
                               T* __restrict__ out, int64_t nout) {
  using WS = FiltTeamWs<T, D>;
  POF_BTEAM_PROLOGUE(WS)
  if (t >= nout) return;
  if (frozen[gp[t]]) return;
  FiltTeamWs<T, D>& w = ws_;
  const int64_t i0 = goff[t], i1 = goff[t + 1];
  t_load_filt<T, TS, D>(tm, in, nin, i0, w.A1, w.b1, w.U1, w.e1, w.Z1);
  for (int64_t i = i0 + 1; i < i1; ++i) {
    t_load_filt<T, TS, D>(tm, in, nin, i, w.A2, w.b2, w.U2, w.e2, w.Z2);
    tm.sync();
    t_filt_combine<T, TS, D>(tm, w);
  }
  tm.sync();
  t_store_filt<T, TS, D>(tm, out, nout, t, w.A1, w.b1, w.U1, w.e1, w.Z1);
}

// Top of the filter: the state before each problem's single top element is
// its x0 (the filtering scan starts from x0, filter.py:23-30).
template <typename T, int D, int TS>
__global__ void kb_filt_top(BView v, const T* __restrict__ x0m, const T* __restrict__ x0L,
                            T* __restrict__ states) {
  using WS = FiltTeamWs<T, D>;
  POF_BTEAM_PROLOGUE(WS)
  (void)ws_;
  if (t >= v.Ba) return;
  const int b = v.ap[t];
  if (v.frozen[b]) return;
  for (int f = tm.r; f < D + D * D; f += TS) {
    const T val = (f < D) ? x0m[(int64_t)b * D + f] : x0L[(int64_t)b * D * D + f - D];
    states[f * v.Ba + t] = val;
  }
}

// Filter down-sweep to level l from level l + 1: states before every element
// of each group from the state before the group.
template <typename T, int D, int TS>
__global__ void kb_filt_down(const int64_t* __restrict__ goff, const int32_t* __restrict__ gp,
                             const int32_t* __restrict__ frozen, const T* __restrict__ elems, int64_t n,
                             const T* __restrict__ states_up, int64_t nup, T* __restrict__ states) {
  using WS = FiltTeamWs<T, D>;
  POF_BTEAM_PROLOGUE(WS)
  if (t >= nup) return;
  if (frozen[gp[t]]) return;
  FiltTeamWs<T, D>& w = ws_;
  const int64_t i0 = goff[t], i1 = goff[t + 1];
  t_load_state<T, TS, D>(tm, states_up, nup, t, w.b1, w.U1);
  tm.sync();
  for (int64_t i = i0; i < i1; ++i) {
    t_store_state<T, TS, D>(tm, states, n, i, w.b1, w.U1);
    tm.sync();
    if (i + 1 < i1) {
      t_load_filt<T, TS, D>(tm, elems, n, i, w.A2, w.b2, w.U2, w.e2, w.Z2);
      tm.sync();
      t_filt_apply<T, TS, D>(tm, w);
    }
  }
}

// Filter level 0, second pass: the Kalman filter over each chunk from the
// state before it, writing filtered states, the smoother elements
// (smoother.py:25-52) and the chunk's sigma^2 / NLL / filter-objective sums.
template <typename T, int D, int DY, int TS>
__global__ void kb_filt_l0_down(BView v, const T* __restrict__ F, const T* __restrict__ QL,
                                const T* __restrict__ H, const T* __restrict__ c, const T* __restrict__ states1,
                                T* __restrict__ means, T* __restrict__ chols, T* __restrict__ selems,
                                double* __restrict__ partials) {
  using WS = L0KFWs<T, D, DY, false>;
  POF_BL0_PROLOGUE(WS, D / DY)
  if (t >= v.n1) return;
  const int b = v.cp[t];
  if (v.frozen[b]) return;
  StepKFWs<T, D, DY>& w = ws_.s;
  using GL = SmoLayout<D>;
  constexpr int L1 = Ld<D>::v, L2 = Ld<2 * D>::v;
  const int64_t s0 = v.cs[t], s1 = v.ce[t];
  const int64_t n = v.n;
  t_load_state<T, TS, D>(tm, states1, v.n1, t, w.m, w.L);
  tm.sync();
  if (s0 == v.gb[b]) {  // first chunk of the problem: its grid point 0 holds x0
    const int64_t g = s0;
    for (int f = tm.r; f < D + D * D; f += TS) {
      if (f < D)
        means[g * D + f] = w.m[f];
      else
        chols[g * D * D + f - D] = w.L[((f - D) / D) * L1 + (f - D) % D];
    }
  }
  double ssq = 0.0, nll = 0.0, fobj = 0.0;
  for (int64_t s = s0; s < s1; ++s) {
    if (!POF_IN(s + 1, v.n)) break;  // writes grid point s + 1
    t_load_step<T, TS, D, DY>(tm, w, H + s * DY * D, c + s * DY, nullptr);
    for (int i = tm.r; i < D; i += TS) ws_.mold[i] = w.m[i];
    tm.sync();
    t_kf_step<T, TS, D, DY, true>(tm, w, fq.F, fq.QL, StepStruct{fq.wq, fq.wf, true});
    ssq += (double)w.sc[0];
    nll += (double)w.sc[1];
    fobj += (double)t_objective<T, TS, D>(tm, fq.F, fq.QLi, ws_.mold, w.m, ws_.r);
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
    const int64_t g = s + 1;
    for (int f = tm.r; f < D + D * D; f += TS) {
      if (f < D)
        means[g * D + f] = w.m[f];
      else
        chols[g * D * D + f - D] = w.L[((f - D) / D) * L1 + (f - D) % D];
    }
    tm.sync();
  }
  if (tm.r == 0) {
    partials[P_SSQ * v.n1 + t] = ssq;
    partials[P_NLL * v.n1 + t] = nll;
    partials[P_FOBJ * v.n1 + t] = fobj;
  }
}

// Smoother level 0: composite of each chunk's smoother elements.
template <typename T, int D, int TS>
__global__ void kb_smo_l0_reduce(BView v, const T* __restrict__ selems, T* __restrict__ out) {
  using WS = SmoTeamWs<T, D>;
  POF_BTEAM_PROLOGUE(WS)
  if (t >= v.n1) return;
  if (v.frozen[v.cp[t]]) return;
  SmoTeamWs<T, D>& w = ws_;
  const int64_t i0 = v.cs[t], i1 = v.ce[t];
  t_load_smo<T, TS, D>(tm, selems, v.n, i0, w.g2, w.E2, w.D2m);
  for (int64_t i = i0 + 1; i < i1; ++i) {
    t_load_smo<T, TS, D>(tm, selems, v.n, i, w.g1, w.E1, w.D1);
    tm.sync();
    t_smooth_combine<T, TS, D>(tm, w);
  }
  tm.sync();
  t_store_smo<T, TS, D>(tm, out, v.n1, t, w.g2, w.E2, w.D2m);
}

template <typename T, int D, int TS>
__global__ void kb_smo_reduce(const int64_t* __restrict__ goff, const int32_t* __restrict__ gp,
                              const int32_t* __restrict__ frozen, const T* __restrict__ in, int64_t nin,
                              T* __restrict__ out, int64_t nout) {
  using WS = SmoTeamWs<T, D>;
  POF_BTEAM_PROLOGUE(WS)
  if (t >= nout) return;
  if (frozen[gp[t]]) return;
  SmoTeamWs<T, D>& w = ws_;
  const int64_t i0 = goff[t], i1 = goff[t + 1];
  t_load_smo<T, TS, D>(tm, in, nin, i0, w.g2, w.E2, w.D2m);
  for (int64_t i = i0 + 1; i < i1; ++i) {
    t_load_smo<T, TS, D>(tm, in, nin, i, w.g1, w.E1, w.D1);
    tm.sync();
    t_smooth_combine<T, TS, D>(tm, w);
  }
  tm.sync();
  t_store_smo<T, TS, D>(tm, out, nout, t, w.g2, w.E2, w.D2m);
}

// Top of the smoother: the state after each problem's single top element is
// its terminal filtered state (the reverse scan starts from the last
// filtering state, smoother.py:14-16).
template <typename T, int D, int TS>
__global__ void kb_smo_top(BView v, const T* __restrict__ means, const T* __restrict__ chols,
                           T* __restrict__ ends) {
  using WS = SmoTeamWs<T, D>;
  POF_BTEAM_PROLOGUE(WS)
  (void)ws_;
  if (t >= v.Ba) return;
  const int b = v.ap[t];
  if (v.frozen[b]) return;
  const int64_t g = v.gb[b] + v.ns[b];
  for (int f = tm.r; f < D + D * D; f += TS) {
    const T val = (f < D) ? means[g * D + f] : chols[g * D * D + f - D];
    ends[f * v.Ba + t] = val;
  }
}

template <typename T, int D, int TS>
__global__ void kb_smo_down(const int64_t* __restrict__ goff, const int32_t* __restrict__ gp,
                            const int32_t* __restrict__ frozen, const T* __restrict__ elems, int64_t n,
                            const T* __restrict__ ends_up, int64_t nup, T* __restrict__ ends) {
  using WS = SmoTeamWs<T, D>;
  POF_BTEAM_PROLOGUE(WS)
  if (t >= nup) return;
  if (frozen[gp[t]]) return;
  SmoTeamWs<T, D>& w = ws_;
  const int64_t i0 = goff[t], i1 = goff[t + 1];
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

// Smoother level 0, second pass: smoothed states of each chunk from the
// state after it, calibrated by the problem's sqrt(sigma^2) when scale is
// given (pof/step.py:42-44), with the chunk's smoother-objective and
// convergence-test sums (convergence_criteria.py:10).
template <typename T, int D, int TS>
__global__ void kb_smo_l0_down(BView v, const T* __restrict__ F, const T* __restrict__ QL,
                               const T* __restrict__ selems, const T* __restrict__ ends1, T* __restrict__ means,
                               T* __restrict__ chols, const double* __restrict__ scale,
                               const T* __restrict__ means_old, double c_mrtol, double c_matol,
                               double* __restrict__ partials) {
  using WS = SmoL0Ws<T, D, false>;
  POF_BL0_PROLOGUE(WS, 0)
  if (t >= v.n1) return;
  const int b = v.cp[t];
  if (v.frozen[b]) return;
  SmoTeamWs<T, D>& w = ws_.s;
  constexpr int L1 = Ld<D>::v;
  const int64_t s0 = v.cs[t], s1 = v.ce[t];
  const T sc = scale ? (T)scale[b] : T(1);
  t_load_state<T, TS, D>(tm, ends1, v.n1, t, w.g1, w.D1);
  tm.sync();
  double sobj = 0.0, notclose = 0.0;
  auto close_count = [&](int64_t g) {
    if (!means_old) return;
    for (int i = tm.r; i < D; i += TS) {
      const double a = (double)means_old[g * D + i], bb = (double)w.g1[i];
      bool ok;
      if (isfinite(a) && isfinite(bb))
        ok = fabs(a - bb) <= c_matol + c_mrtol * fabs(bb);
      else
        ok = (a == bb);
      notclose += ok ? 0.0 : 1.0;
    }
  };
  if (s1 == v.gb[b] + v.ns[b]) {  // last chunk: the terminal grid point
    const int64_t g = s1;
    close_count(g);
    if (scale)
      for (int f = tm.r; f < D * D; f += TS) chols[g * D * D + f] = w.D1[(f / D) * L1 + f % D] * sc;
  }
  for (int64_t k = s1 - 1; k >= s0; --k) {
    if (!POF_IN(k, v.n)) break;
    for (int i = tm.r; i < D; i += TS) ws_.mnext[i] = w.g1[i];
    t_load_smo<T, TS, D>(tm, selems, v.n, k, w.g2, w.E2, w.D2m);
    tm.sync();
    t_smooth_apply<T, TS, D>(tm, w);
    sobj += (double)t_objective<T, TS, D>(tm, fq.F, fq.QLi, w.g1, ws_.mnext, ws_.r);
    const int64_t g = k;
    close_count(g);
    for (int f = tm.r; f < D + D * D; f += TS) {
      if (f < D)
        means[g * D + f] = w.g1[f];
      else
        chols[g * D * D + f - D] = w.D1[((f - D) / D) * L1 + (f - D) % D] * sc;
    }
    tm.sync();
  }
  notclose = (double)tm.sum(notclose);
  if (tm.r == 0) {
    partials[P_SOBJ * v.n1 + t] = sobj;
    partials[P_NOTCLOSE * v.n1 + t] = notclose;
  }
}

#undef POF_BTEAM_PROLOGUE
#undef POF_BL0_PROLOGUE

// Fixed-order sum of a problem's chunk partials over [c0, c1) by one warp:
// lane l sums chunks c0 + l, c0 + l + 32, ... in order, then a fixed
// butterfly; every lane returns the total.
__device__ __forceinline__ double warp_chunk_sum(const double* __restrict__ x, int64_t c0, int64_t c1, int lane) {
  double s = 0.0;
  for (int64_t i = c0 + lane; i < c1; i += 32) s += x[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// After the filter: each active problem's sigma^2 (filter.py:105-114), NLL
// and filter objective; one warp per problem.
static __global__ void kb_fin_filter(BView v, const double* __restrict__ partials, int DY, double* __restrict__ pscal,
                                     double* __restrict__ pscale) {
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (k >= v.Ba) return;
  const int b = v.ap[k];
  if (v.frozen[b]) return;
  const int64_t c0 = v.pc[k], c1 = v.pc[k + 1];
  const double ssq = warp_chunk_sum(partials + P_SSQ * v.n1, c0, c1, lane);
  const double nll = warp_chunk_sum(partials + P_NLL * v.n1, c0, c1, lane);
  const double fobj = warp_chunk_sum(partials + P_FOBJ * v.n1, c0, c1, lane);
  if (lane == 0) {
    const double nb = (double)v.ns[b];
    const double s = ssq / nb / (double)DY;
    double* sc = pscal + (int64_t)kBatchScalars * b;
    sc[S_SSQ] = s;
    sc[S_NLL] = nll;
    sc[S_FOBJ] = fobj;
    pscale[b] = sqrt(s);
  }
}

// After the smoother: objective, then the loop control of
// pof/solver.py:36-57 with crit of convergence_criteria.py:4-13 per problem
// (the rule of k_ieks_control), freezing the problems that stop.  nactive
// counts the problems that go on.
static __global__ void kb_control(BView v, const double* __restrict__ partials, double* __restrict__ pscal,
                                  int32_t* __restrict__ frozen, int64_t maxiters, double rtol, double atol,
                                  int32_t* __restrict__ nactive) {
  const int64_t k = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (k >= v.Ba) return;
  const int b = v.ap[k];
  if (frozen[b]) return;
  const int64_t c0 = v.pc[k], c1 = v.pc[k + 1];
  const double sobj = warp_chunk_sum(partials + P_SOBJ * v.n1, c0, c1, lane);
  const double nc = warp_chunk_sum(partials + P_NOTCLOSE * v.n1, c0, c1, lane);
  if (lane != 0) return;
  double* sc = pscal + (int64_t)kBatchScalars * b;
  sc[S_OBJ] = sobj;
  sc[S_NOTCLOSE] = nc;
  const double it = sc[S_ITER] + 1.0;
  sc[S_ITER] = it;
  const double obj = sobj, nll = sc[S_NLL], oo = sc[S_OBJ_OLD];
  const bool nan = isnan(obj) || isnan(nll);
  if (v.rtol) rtol = v.rtol[b];
  if (v.maxit) maxiters = v.maxit[b];
  bool objc;
  if (isfinite(oo) && isfinite(obj))
    objc = fabs(oo - obj) <= atol + rtol * fabs(obj);
  else
    objc = (oo == obj);
  const bool conv = nan || objc || nc == 0.0;
  const bool cancelled = v.cancel && v.cancel[b] != 0;
  const bool cont = !conv && it <= (double)maxiters && !cancelled;
  sc[S_OBJ_OLD] = obj;
  sc[S_NLL_OLD] = nll;
  sc[S_CONT] = cont ? 1.0 : 0.0;
  sc[S_STATUS] = (cancelled && !conv) ? (double)POF_SOLVE_CANCELLED : stop_status(conv, obj, nll);
  if (cont)
    atomicAdd(nactive, 1);
  else
    frozen[b] = 1;
}

// End of a batched solve, one block per problem: the latest iterate into
// `means` (it sits in the second buffer after an odd number of
// iterations), the final calibration of the returned chol
// (pof/solver.py:66-69), and info[b] = (iterations, nll, obj, sigma^2).
template <typename T>
__global__ void kb_finish(const int64_t* __restrict__ gb, const int64_t* __restrict__ ns,
                          const double* __restrict__ pscal, const double* __restrict__ pscale, int D, int calibrate,
                          T* __restrict__ means, const T* __restrict__ means2, T* __restrict__ chols,
                          double* __restrict__ info) {
  const int b = blockIdx.x;
  const double* sc = pscal + (int64_t)kBatchScalars * b;
  const int64_t g0 = gb[b], g1 = gb[b] + ns[b] + 1;
  const long long it = (long long)sc[S_ITER];
  if (it & 1)
    for (int64_t i = g0 * D + threadIdx.x; i < g1 * D; i += blockDim.x) means[i] = means2[i];
  if (calibrate) {
    const T s = (T)pscale[b];
    for (int64_t i = g0 * D * D + threadIdx.x; i < g1 * D * D; i += blockDim.x) chols[i] *= s;
  }
  if (info && threadIdx.x == 0) {
    double* o = info + (int64_t)POF_I_COUNT * b;
    o[POF_I_ITERATIONS] = sc[S_ITER];
    o[POF_I_NLL] = sc[S_NLL];
    o[POF_I_OBJ] = sc[S_OBJ];
    o[POF_I_SSQ] = sc[S_SSQ];
    o[POF_I_STATUS] = sc[S_STATUS];
  }
}

// ---------------------------------------------------------------------------
// Mixed precision (float32 iterations, float64 polish) for a batch: the
// per-problem form of pof_ieks_solve_mixed's float32 phase.
// ---------------------------------------------------------------------------

// EK1 linearization in float64 at the float64 iterate (kb_linearize's
// arithmetic), each row of (H, c) scaled to unit norm and rounded to float32
// (a noiseless observation row can be scaled freely; k_rows_to_f32).
template <int D, int DY>
__global__ void kb_lin_mixed(BView v, const double* __restrict__ params, const double* __restrict__ means,
                             float* __restrict__ H, float* __restrict__ c) {
  constexpr int Q1 = D / DY;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t t = i / v.C0;
  if (t >= v.n1) return;
  const int b = v.cp[t];
  if (v.frozen[b]) return;
  const int64_t s = v.cs[t] + i % v.C0;
  if (s >= v.ce[t]) return;
  const double p0 = v.p01[2 * b], p1 = v.p01[2 * b + 1];
  const double* m = means + (s + 1) * D;
  double y[DY], f[DY], J[DY * DY];
#pragma unroll
  for (int k = 0; k < DY; ++k) y[k] = p0 * m[k * Q1];
  field_eval<double, DY>(v.fld[b], params + 4 * b, y, f, J);
#pragma unroll
  for (int r = 0; r < DY; ++r) {
    double h[D];
#pragma unroll
    for (int k = 0; k < D; ++k) h[k] = 0.0;
#pragma unroll
    for (int j = 0; j < DY; ++j) h[j * Q1] = -(J[r * DY + j] * p0);
    h[r * Q1 + 1] += p1;
    const double res = p1 * m[r * Q1 + 1] - f[r];
    double hm = 0.0, ss = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) hm = fma(h[k], m[k], hm);
#pragma unroll
    for (int k = 0; k < D; ++k) ss = fma(h[k], h[k], ss);
    const double inv = ss > 0.0 ? 1.0 / sqrt(ss) : 1.0;
#pragma unroll
    for (int k = 0; k < D; ++k) H[(s * DY + r) * D + k] = (float)(h[k] * inv);
    c[s * DY + r] = (float)((res - hm) * inv);
  }
}

template <int D, int DY>
void batch_lin_mixed(const BView& v, const double* params, const double* means, float* H, float* c, cudaStream_t st) {
  ProfScope ps(PK_LINEARIZE, st);
  kb_lin_mixed<D, DY><<<grid_for(v.n1 * v.C0, 128), 128, 0, st>>>(v, params, means, H, c);
}

// Per-problem state of the float32 phase (doubles): iterations kept, best
// and previous relative change, consecutive non-shrinking count, this
// iteration's max |dy|, max |y|, non-finite flag, accept flag.
enum Mixed32 : int { M_IT = 0, M_BEST, M_PREV, M_WORSE, M_DY, M_AY, M_BAD, M_ACCEPT, M_COUNT = 8 };

// max |y_new - y_old| and max |y_old| over the problem's projected states
// y = p0 m[i (q+1)] (the float32 candidate against the float64 iterate) and
// a non-finite flag; one block per active problem (k_ychange per problem).
template <int D, int DY>
__global__ void kb_ychange(BView v, const float* __restrict__ mnew, const double* __restrict__ mold,
                           double* __restrict__ mst) {
  constexpr int Q1 = D / DY;
  const int64_t k = blockIdx.x;
  const int b = v.ap[k];
  if (v.frozen[b]) return;
  const double p0 = v.p01[2 * b];
  const int64_t g0 = v.gb[b], g1 = v.gb[b] + v.ns[b] + 1;
  double dy = 0.0, ay = 0.0;
  int bad = 0;
  for (int64_t idx = g0 * DY + threadIdx.x; idx < g1 * DY; idx += blockDim.x) {
    const int64_t g = idx / DY;
    const int i = (int)(idx % DY);
    const double a = (double)mnew[g * D + i * Q1], o = mold[g * D + i * Q1];
    bad |= !isfinite(a);
    dy = fmax(dy, fabs(p0 * (a - o)));
    ay = fmax(ay, fabs(p0 * o));
  }
  __shared__ double sdy[32], say[32];
  __shared__ int sbad[32];
  for (int o = 16; o > 0; o >>= 1) {
    dy = fmax(dy, __shfl_xor_sync(0xffffffffu, dy, o));
    ay = fmax(ay, __shfl_xor_sync(0xffffffffu, ay, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sdy[w] = dy;
    say[w] = ay;
    sbad[w] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 1; j < nw; ++j) {
      dy = fmax(dy, sdy[j]);
      ay = fmax(ay, say[j]);
      bad |= sbad[j];
    }
    double* m = mst + (int64_t)M_COUNT * b;
    m[M_DY] = dy;
    m[M_AY] = ay;
    m[M_BAD] = bad ? 1.0 : 0.0;
  }
}

// The float32 phase's stopping rules per problem (pof_ieks_solve_mixed):
// a non-finite candidate is dropped and ends the phase; otherwise it is
// kept; the phase ends when the relative change is below rtol_f32, after
// three changes in a row that did not shrink (counted once the smallest
// change is below settle_f32), or after maxiters_f32 kept iterations.
// done32 marks the problems whose phase has ended.
static __global__ void kb_ctl32(BView v, double* __restrict__ mst, int32_t* __restrict__ done32, int64_t maxiters_f32,
                                double rtol_f32, double settle_f32, int32_t* __restrict__ nactive) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= v.Ba) return;
  const int b = v.ap[k];
  if (done32[b]) return;
  double* m = mst + (int64_t)M_COUNT * b;
  if (m[M_BAD] != 0.0 || (v.cancel && v.cancel[b] != 0)) {  // non-finite candidate, or a cancelled request
    m[M_ACCEPT] = 0.0;
    done32[b] = 1;
    return;
  }
  m[M_ACCEPT] = 1.0;
  m[M_IT] += 1.0;
  const double rel = m[M_AY] > 0.0 ? m[M_DY] / m[M_AY] : m[M_DY];
  m[M_BEST] = rel < m[M_BEST] ? rel : m[M_BEST];
  bool stop = rel < rtol_f32;
  // non-shrinking changes count once the smallest change is below settle_f32
  if (rel >= m[M_PREV])
    m[M_WORSE] += m[M_BEST] < settle_f32 ? 1.0 : 0.0;
  else
    m[M_WORSE] = 0.0;
  stop = stop || m[M_WORSE] >= 3.0 || m[M_IT] >= (double)maxiters_f32;
  m[M_PREV] = rel;
  if (stop)
    done32[b] = 1;
  else
    atomicAdd(nactive, 1);
}

// Kept candidates become the float64 iterate; one block per active problem.
template <int D>
__global__ void kb_accept(BView v, const float* __restrict__ mnew, double* __restrict__ means,
                          const double* __restrict__ mst) {
  const int b = v.ap[blockIdx.x];
  if (mst[(int64_t)M_COUNT * b + M_ACCEPT] == 0.0) return;
  const int64_t g0 = v.gb[b], g1 = v.gb[b] + v.ns[b] + 1;
  for (int64_t i = g0 * D + threadIdx.x; i < g1 * D; i += blockDim.x) means[i] = (double)mnew[i];
}

// End of the float32 phase: a problem whose best relative change never came
// within 100 rtol_f32 (float32 too coarse for it) goes back to its input
// trajectory, with no float32 iterations counted; one block per problem.
template <int D>
__global__ void kb_revert(const int64_t* __restrict__ gb, const int64_t* __restrict__ ns, double* __restrict__ mst,
                          double rtol_f32, const double* __restrict__ keep, double* __restrict__ means) {
  const int b = blockIdx.x;
  double* m = mst + (int64_t)M_COUNT * b;
  if (!(m[M_IT] > 0.0) || m[M_BEST] < 100.0 * rtol_f32) return;
  const int64_t g0 = gb[b], g1 = gb[b] + ns[b] + 1;
  for (int64_t i = g0 * D + threadIdx.x; i < g1 * D; i += blockDim.x) means[i] = keep[i];
  __syncthreads();
  if (threadIdx.x == 0) m[M_IT] = 0.0;
}

template <int D, int DY>
void batch_ychange(const BView& v, const float* mnew, const double* mold, double* mst, cudaStream_t st) {
  kb_ychange<D, DY><<<(unsigned)v.Ba, 256, 0, st>>>(v, mnew, mold, mst);
}
template <int D>
void batch_accept(const BView& v, const float* mnew, double* means, const double* mst, cudaStream_t st) {
  kb_accept<D><<<(unsigned)v.Ba, 256, 0, st>>>(v, mnew, means, mst);
}
template <int D>
void batch_revert(int64_t B, const int64_t* gb, const int64_t* ns, double* mst, double rtol_f32, const double* keep,
                  double* means, cudaStream_t st) {
  kb_revert<D><<<(unsigned)B, 256, 0, st>>>(gb, ns, mst, rtol_f32, keep, means);
}

static __global__ void kb_init_mixed(double* __restrict__ mst, int64_t B) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= B * M_COUNT) return;
  const int f = (int)(i % M_COUNT);
  mst[i] = (f == M_BEST || f == M_PREV) ? 1e300 : 0.0;
}

static __global__ void kb_d2f(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

// Type-erased arguments of one batched iteration (pointers of the plan's
// element type T).
struct BatchRaw {
  BView v;
  const BatchLevels* L;
  char* lw;  // level part of the workspace
  const void* params;  // (B, 4)
  const void* x0m;     // (B, D)
  const void* x0L;     // (B, D, D)
  const void* F;
  const void* QL;
  void* H;
  void* c;
  void* selem;
  void* chols;
  double* pscal;
  double* pscale;
  int32_t* frozen;
  int32_t* nactive;
  int64_t maxiters;
  double rtol, atol, mrtol, matol;
  bool calibrate;
  int team;  // level-0 lanes
};

// Launch sequence of one IEKS iteration of a plan, for one (T, D, DY).
template <typename T, int D, int DY>
struct BatchDriver {
  static constexpr int TSW = TeamSize<D>::v;
  static constexpr int TSN = TSW / 2 >= 4 ? TSW / 2 : 4;
  using FWS = FiltTeamWs<T, D>;
  using SWS = SmoTeamWs<T, D>;
  template <int TS, typename WS, typename... KArgs, typename... Args>
  static void launch_l0(void (*kern)(KArgs...), int64_t nteams, cudaStream_t st, Args... args) {
    using B = TeamBlockH<WS, TS, FQHeader<T, D, false>::bytes>;
    kern<<<(unsigned)((nteams + B::teams - 1) / B::teams), B::threads, B::smem, st>>>(args...);
  }

  template <typename U>
  static U* at(char* base, size_t off) {
    return reinterpret_cast<U*>(base + off);
  }

  // One IEKS iteration: linearize at mold, filter and smooth into mnew,
  // then the convergence test of every problem against mold.
  static void iteration(const BatchRaw& a, const void* mold, void* mnew, cudaStream_t st) {
    cudaMemsetAsync(a.nactive, 0, sizeof(int32_t), st);
    {
      ProfScope ps(PK_LINEARIZE, st);
      kb_linearize<T, D, DY><<<grid_for(a.v.n1 * a.v.C0, 128), 128, 0, st>>>(
          a.v, static_cast<const T*>(a.params), static_cast<const T*>(mold), static_cast<T*>(a.H),
          static_cast<T*>(a.c));
    }
    filtsmooth(a, mold, mnew, st);
    {
      ProfScope ps(PK_CONTROL, st);
      kb_control<<<grid_for(a.v.Ba * 32, 128), 128, 0, st>>>(a.v, at<double>(a.lw, a.L->partials), a.pscal,
                                                            a.frozen, a.maxiters, a.rtol, a.atol, a.nactive);
    }
  }

  // Filter and smoother of the linear model in a.H, a.c (per-problem
  // sigma^2 / NLL / objective sums into a.pscal; not-close counts against
  // mold when given).
  static void filtsmooth(const BatchRaw& a, const void* mold, void* mnew, cudaStream_t st) {
    if (a.team == TSN && TSN != TSW)
      filtsmooth_ts<TSN>(a, static_cast<const T*>(mold), static_cast<T*>(mnew), st);
    else
      filtsmooth_ts<TSW>(a, static_cast<const T*>(mold), static_cast<T*>(mnew), st);
  }

  template <int TS>
  static void filtsmooth_ts(const BatchRaw& a, const T* mold, T* mnew, cudaStream_t st) {
    constexpr int TU = TSW;
    const BatchLevels& L = *a.L;
    const BView& v = a.v;
    char* lw = a.lw;
    const int64_t n1 = v.n1;
    const T* x0m = static_cast<const T*>(a.x0m);
    const T* x0L = static_cast<const T*>(a.x0L);
    const T* F = static_cast<const T*>(a.F);
    const T* QL = static_cast<const T*>(a.QL);
    T* H = static_cast<T*>(a.H);
    T* c = static_cast<T*>(a.c);
    T* selem = static_cast<T*>(a.selem);
    T* chols = static_cast<T*>(a.chols);
    const int32_t* frozen = a.frozen;
    {
      ProfScope ps(PK_FILT_L0_REDUCE, st);
      launch_l0<TS, L0FoldWs<T, D, DY, false>>(kb_filt_l0_reduce<T, D, DY, TS>, n1, st, v, F, QL, (const T*)H,
                                               (const T*)c, at<T>(lw, L.felem[1]));
    }
    for (int l = 2; l <= L.nlev; ++l) {
      ProfScope ps(PK_FILT_REDUCE, st);
      launch_team<FWS, TU>(kb_filt_reduce<T, D, TU>, L.cnt[l], st, (const int64_t*)at<int64_t>(lw, L.goff[l]),
                           (const int32_t*)at<int32_t>(lw, L.gp[l]), frozen, (const T*)at<T>(lw, L.felem[l - 1]),
                           L.cnt[l - 1], at<T>(lw, L.felem[l]), L.cnt[l]);
    }
    {
      ProfScope ps(PK_FILT_TOP, st);
      launch_team<FWS, TU>(kb_filt_top<T, D, TU>, v.Ba, st, v, x0m, x0L, at<T>(lw, L.fstate[L.nlev]));
    }
    for (int l = L.nlev - 1; l >= 1; --l) {
      ProfScope ps(PK_FILT_DOWN, st);
      launch_team<FWS, TU>(kb_filt_down<T, D, TU>, L.cnt[l + 1], st, (const int64_t*)at<int64_t>(lw, L.goff[l + 1]),
                           (const int32_t*)at<int32_t>(lw, L.gp[l + 1]), frozen, (const T*)at<T>(lw, L.felem[l]),
                           L.cnt[l], (const T*)at<T>(lw, L.fstate[l + 1]), L.cnt[l + 1], at<T>(lw, L.fstate[l]));
    }
    {
      ProfScope ps(PK_FILT_L0_DOWN, st);
      launch_l0<TS, L0KFWs<T, D, DY, false>>(kb_filt_l0_down<T, D, DY, TS>, n1, st, v, F, QL, (const T*)H,
                                             (const T*)c, (const T*)at<T>(lw, L.fstate[1]), mnew, chols, selem,
                                             at<double>(lw, L.partials));
    }
    {
      ProfScope ps(PK_FILT_FINALIZE, st);
      kb_fin_filter<<<grid_for(v.Ba * 32, 128), 128, 0, st>>>(v, at<double>(lw, L.partials), DY, a.pscal, a.pscale);
    }
    {
      ProfScope ps(PK_SMO_L0_REDUCE, st);
      launch_team<SWS, TS>(kb_smo_l0_reduce<T, D, TS>, n1, st, v, (const T*)selem, at<T>(lw, L.gelem[1]));
    }
    for (int l = 2; l <= L.nlev; ++l) {
      ProfScope ps(PK_SMO_REDUCE, st);
      launch_team<SWS, TU>(kb_smo_reduce<T, D, TU>, L.cnt[l], st, (const int64_t*)at<int64_t>(lw, L.goff[l]),
                           (const int32_t*)at<int32_t>(lw, L.gp[l]), frozen, (const T*)at<T>(lw, L.gelem[l - 1]),
                           L.cnt[l - 1], at<T>(lw, L.gelem[l]), L.cnt[l]);
    }
    {
      ProfScope ps(PK_SMO_TOP, st);
      launch_team<SWS, TU>(kb_smo_top<T, D, TU>, v.Ba, st, v, (const T*)mnew, (const T*)chols,
                           at<T>(lw, L.gend[L.nlev]));
    }
    for (int l = L.nlev - 1; l >= 1; --l) {
      ProfScope ps(PK_SMO_DOWN, st);
      launch_team<SWS, TU>(kb_smo_down<T, D, TU>, L.cnt[l + 1], st, (const int64_t*)at<int64_t>(lw, L.goff[l + 1]),
                           (const int32_t*)at<int32_t>(lw, L.gp[l + 1]), frozen, (const T*)at<T>(lw, L.gelem[l]),
                           L.cnt[l], (const T*)at<T>(lw, L.gend[l + 1]), L.cnt[l + 1], at<T>(lw, L.gend[l]));
    }
    {
      ProfScope ps(PK_SMO_L0_DOWN, st);
      launch_l0<TS, SmoL0Ws<T, D, false>>(kb_smo_l0_down<T, D, TS>, n1, st, v, F, QL, (const T*)selem,
                                          (const T*)at<T>(lw, L.gend[1]), mnew, chols,
                                          a.calibrate ? (const double*)a.pscale : nullptr, mold, a.mrtol, a.matol,
                                          at<double>(lw, L.partials));
    }
  }

  static void finish(int64_t B, const int64_t* gb, const int64_t* ns, const double* pscal, const double* pscale,
                     bool calibrate, void* means, const void* means2, void* chols, double* info, cudaStream_t st) {
    kb_finish<T><<<(unsigned)B, 256, 0, st>>>(gb, ns, pscal, pscale, D, calibrate ? 1 : 0, static_cast<T*>(means),
                                              static_cast<const T*>(means2), static_cast<T*>(chols), info);
  }
};

struct BatchOps {
  void (*iteration)(const BatchRaw&, const void*, void*, cudaStream_t);
  void (*filtsmooth)(const BatchRaw&, const void*, void*, cudaStream_t);
  void (*finish)(int64_t, const int64_t*, const int64_t*, const double*, const double*, bool, void*, const void*,
                 void*, double*, cudaStream_t);
  // float32 phase of the mixed-precision batch (float32 table only):
  // float64 linearization at the float64 iterate into float32 rows
  void (*lin_mixed)(const BView&, const double*, const double*, float*, float*, cudaStream_t);
  void (*ychange)(const BView&, const float*, const double*, double*, cudaStream_t);
  void (*accept)(const BView&, const float*, double*, const double*, cudaStream_t);
  void (*revert)(int64_t, const int64_t*, const int64_t*, double*, double, const double*, double*, cudaStream_t);
  int tsn, tsw;  // level-0 team sizes available (narrow, wide)
};

template <typename T, int D, int DY>
const BatchOps* batch_ops_impl() {
  static const BatchOps ops{&BatchDriver<T, D, DY>::iteration, &BatchDriver<T, D, DY>::filtsmooth,
                            &BatchDriver<T, D, DY>::finish, &batch_lin_mixed<D, DY>, &batch_ychange<D, DY>,
                            &batch_accept<D>, &batch_revert<D>, BatchDriver<T, D, DY>::TSN,
                            BatchDriver<T, D, DY>::TSW};
  return &ops;
}

// One specialization per compiled batch shape (pof_binst_D<D>_d<d>.cu).
template <int D, int DY>
const BatchOps* batch_ops_shape(int dtype);

const BatchOps* find_batch_shape(int dtype, int D, int DY);

}  // namespace pof
