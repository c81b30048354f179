// Host-side orchestration of the chunked filter/smoother for one (T, D, DY):
// kernel launches in stream order over a caller-provided workspace.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "../../include/pof.h"
#include "pof_kernels.cuh"
#include "pof_team_kernels.cuh"
#include "pof_plan.h"
#include "pof_prof.h"

namespace pof {

enum Scalar : int {
  S_NLL = 0, S_OBJ = 1, S_SSQ = 2, S_FOBJ = 3, S_NOTCLOSE = 4,
  S_OBJ_OLD = 5, S_NLL_OLD = 6, S_ITER = 7, S_CONT = 8, S_STATUS = 9, S_COUNT = 16
};

// Why a loop that stops now stops (POF_SOLVE_*): the reference's stopping
// rule is unchanged, this only labels it.  Infinite values stop the
// reference's loop through isclose(inf, inf), so they are reported with NaN.
__device__ __forceinline__ double stop_status(bool conv, double obj, double nll) {
  if (!isfinite(obj) || !isfinite(nll)) return (double)POF_SOLVE_NONFINITE;
  return conv ? (double)POF_SOLVE_CONVERGED : (double)POF_SOLVE_MAXITERS;
}

template <typename T>
__global__ void k_finalize_filter(const double* __restrict__ partials, int64_t n1, int64_t n, int DY,
                                  double* __restrict__ scalars, T* __restrict__ scale) {
  const double ssq = block_sum_fixed<256>(partials + P_SSQ * n1, n1);
  const double nll = block_sum_fixed<256>(partials + P_NLL * n1, n1);
  const double fobj = block_sum_fixed<256>(partials + P_FOBJ * n1, n1);
  if (threadIdx.x == 0) {
    const double s = ssq / (double)n / (double)DY;
    scalars[S_SSQ] = s;
    scalars[S_NLL] = nll;
    scalars[S_FOBJ] = fobj;
    *scale = (T)sqrt(s);
  }
}

static __global__ void k_finalize_smoother(const double* __restrict__ partials, int64_t n1, double* __restrict__ scalars) {
  const double sobj = block_sum_fixed<256>(partials + P_SOBJ * n1, n1);
  const double nc = block_sum_fixed<256>(partials + P_NOTCLOSE * n1, n1);
  if (threadIdx.x == 0) {
    scalars[S_OBJ] = sobj;
    scalars[S_NOTCLOSE] = nc;
  }
}

// Loop control of pof/solver.py:36-57 after one more ieks_step:
// crit (pof/convergence_criteria.py:4-13): stop on NaN, on
// isclose(obj_old, obj, rtol, atol) or when every mean is
// isclose(old, new, mrtol, matol); the reference's values are rtol = 1e-6,
// atol = 1e-9, mrtol = 1e-13, matol = 1e-8.
__device__ __forceinline__ bool ieks_control(double* __restrict__ scalars, int64_t maxiters, double rtol,
                                             double atol) {
  const double k = scalars[S_ITER] + 1.0;
  scalars[S_ITER] = k;
  const double obj = scalars[S_OBJ], nll = scalars[S_NLL];
  const double oo = scalars[S_OBJ_OLD];
  const bool nan = isnan(obj) || isnan(nll);
  bool objc;
  if (isfinite(oo) && isfinite(obj))
    objc = fabs(oo - obj) <= atol + rtol * fabs(obj);
  else
    objc = (oo == obj);
  const bool meansc = scalars[S_NOTCLOSE] == 0.0;
  const bool conv = nan || objc || meansc;
  const bool cont = (k < 1.0) || (!conv && k <= (double)maxiters);
  scalars[S_CONT] = cont ? 1.0 : 0.0;
  scalars[S_STATUS] = stop_status(conv, obj, nll);
  scalars[S_OBJ_OLD] = obj;
  scalars[S_NLL_OLD] = nll;
  return cont;
}

static __global__ void k_ieks_control(double* __restrict__ scalars, int64_t maxiters, double rtol, double atol) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  ieks_control(scalars, maxiters, rtol, atol);
}

// The same control as the last node of the body of a CUDA graph's while
// loop: the loop goes on while the handle is non-zero.  Every iteration adds
// one to the iteration count and the loop stops once it exceeds maxiters + 1
// at the latest, so the while loop ends.
static __global__ void k_ieks_control_graph(double* __restrict__ scalars, int64_t maxiters, double rtol,
                                            double atol, cudaGraphConditionalHandle handle) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const bool cont = ieks_control(scalars, maxiters, rtol, atol);
  cudaGraphSetConditional(handle, cont ? 1u : 0u);
}

static __global__ void k_init_scalars(double* __restrict__ scalars) {
  if (threadIdx.x < S_COUNT) scalars[threadIdx.x] = 0.0;
}

template <typename T>
__global__ void k_scale_inplace(T* __restrict__ x, int64_t count, const T* __restrict__ scale) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < count) x[i] *= *scale;
}

static __global__ void k_copy_scalars(const double* __restrict__ src, double* __restrict__ dst, int which) {
  if (threadIdx.x != 0) return;
  if (which == 0) {  // out_scalars of the filter/smoother entry points
    dst[0] = src[S_NLL];
    dst[1] = src[S_OBJ];
    dst[2] = src[S_SSQ];
    dst[3] = src[S_FOBJ];
    dst[4] = src[S_NOTCLOSE];
  } else {  // info of the solver
    dst[POF_I_ITERATIONS] = src[S_ITER];
    dst[POF_I_NLL] = src[S_NLL];
    dst[POF_I_OBJ] = src[S_OBJ];
    dst[POF_I_SSQ] = src[S_SSQ];
    dst[POF_I_STATUS] = src[S_STATUS];
  }
}

inline unsigned grid_for(int64_t count, int block) { return (unsigned)((count + block - 1) / block); }

// Brackets one launch with profiler events when profiling is on.
struct ProfScope {
  int kind;
  cudaStream_t st;
  ProfScope(int k, cudaStream_t s) : kind(k), st(s) {
    if (prof_on()) prof_begin(kind, st);
  }
  ~ProfScope() {
    if (prof_on()) prof_end(kind, st);
  }
};

// Launch a team kernel over `nteams` teams (TeamBlock teams per block, one
// shared-memory workspace per team).
template <typename WS, int TS, typename... KArgs, typename... Args>
inline void launch_team(void (*kern)(KArgs...), int64_t nteams, cudaStream_t st, Args... args) {
  using B = TeamBlock<WS, TS>;
  const unsigned grid = (unsigned)((nteams + B::teams - 1) / B::teams);
  kern<<<grid, B::threads, B::teams * sizeof(WS), st>>>(args...);
}

// Upper-level launches with few combines (at most this many lanes of wide
// teams) use the wide teams: they are latency-bound, and a wider team
// shortens each combine's chain of FP64 instructions (t_tria's column
// phases, more outputs per t_mm step).  POF_WIDE_LANES overrides.
int wide_lane_limit();

template <typename T, int D, int DY>
struct Driver {
  static constexpr int kBlock = 64;
  static constexpr int TSW = TeamSize<D>::v;                     // wide teams
  static constexpr int TSN = TSW / 2 >= 4 ? TSW / 2 : 4;          // narrow teams
  static constexpr int TSX = TSW < 32 ? 2 * TSW : 32;             // widest teams (latency-bound levels)
  static constexpr bool kTeamL0 = D >= 6;  // pof_plan.h l0_lanes
  using FWS = FiltTeamWs<T, D>;
  using SWS = SmoTeamWs<T, D>;

  // level-0 team kernels: block-shared transition model unless it varies
  // per step (PS)
  template <int TS, bool PS, typename WS, typename... KArgs, typename... Args>
  static void launch_l0(void (*kern)(KArgs...), int64_t nteams, cudaStream_t st, Args... args) {
    using B = TeamBlockH<WS, TS, FQHeader<T, D, PS>::bytes>;
    const unsigned grid = (unsigned)((nteams + B::teams - 1) / B::teams);
    kern<<<grid, B::threads, B::smem, st>>>(args...);
  }

  static void filter(const Plan& p, char* ws, const StepModel& sm, const T* x0m, const T* x0L, T* means, T* chols,
                     cudaStream_t st) {
    if (p.team == TSN && TSN != TSW)
      filter_ts<TSN, TSW>(p, ws, sm, x0m, x0L, means, chols, st);
    else
      filter_ts<TSW, TSW>(p, ws, sm, x0m, x0L, means, chols, st);
  }
  static void smoother(const Plan& p, char* ws, const T* F, const T* QL, int64_t ft_stride, T* means, T* chols,
                       bool calibrate, const T* means_old, cudaStream_t st) {
    if (p.team == TSN && TSN != TSW)
      smoother_ts<TSN, TSW>(p, ws, F, QL, ft_stride, means, chols, calibrate, means_old, st);
    else
      smoother_ts<TSW, TSW>(p, ws, F, QL, ft_stride, means, chols, calibrate, means_old, st);
  }

  struct Bufs {
    char* ws;
    const Plan* p;
    template <typename U>
    U* at(size_t off) const {
      return reinterpret_cast<U*>(ws + off);
    }
  };

  // Filter (phases 1-3) then finalize.  Leaves filtered states in means/chols
  // and the smoother elements in the workspace.
  template <int TS, int TU>
  static void filter_ts(const Plan& p, char* ws, const StepModel& sm, const T* x0m, const T* x0L, T* means,
                        T* chols, cudaStream_t st) {
    Bufs b{ws, &p};
    const int64_t n = p.n;
    const int64_t n1 = p.cnt[1];
    // One chunk (a plan whose level 0 spans the trajectory: the sequential
    // filter): its start state is x0, which the top writes without reading
    // any element, so the chunk's element is not built.
    if (n1 > 1 || p.ks) {
      ProfScope ps(PK_FILT_L0_REDUCE, st);
      if constexpr (kTeamL0) {
        if (sm.ft_stride)
          launch_l0<TS, true, L0FoldWs<T, D, DY, true>>(k_filt_l0_reduce_team<T, D, DY, TS, true>, n1, st, n, p.C0,
                                                        sm, x0m, x0L, b.template at<T>(p.felem[1]), n1);
        else
          launch_l0<TS, false, L0FoldWs<T, D, DY, false>>(k_filt_l0_reduce_team<T, D, DY, TS, false>, n1, st, n,
                                                          p.C0, sm, x0m, x0L, b.template at<T>(p.felem[1]), n1);
      }
      else
        k_filt_l0_reduce<T, D, DY><<<grid_for(n1, kBlock), kBlock, 0, st>>>(n, p.C0, sm, x0m, x0L,
                                                                             b.template at<T>(p.felem[1]), n1);
    }
    const int64_t wide = wide_lane_limit() / TSX;  // teams up to which the widest teams run
    for (int l = 1; l < p.nlev; ++l) {
      ProfScope ps(PK_FILT_REDUCE, st);
      if (p.cnt[l + 1] <= wide)
        launch_team<FWS, TSX>(k_filt_reduce_team<T, D, TSX>, p.cnt[l + 1], st,
                              (const T*)b.template at<T>(p.felem[l]), p.cnt[l], p.Cg,
                              b.template at<T>(p.felem[l + 1]), p.cnt[l + 1]);
      else
        launch_team<FWS, TU>(k_filt_reduce_team<T, D, TU>, p.cnt[l + 1], st, (const T*)b.template at<T>(p.felem[l]),
                             p.cnt[l], p.Cg, b.template at<T>(p.felem[l + 1]), p.cnt[l + 1]);
    }
    if (p.ks) {
      // parallel scan of the top level, ping-ponging between its element
      // buffer and ksbuf; the last step writes the states
      const int64_t K = p.cnt[p.nlev];
      T* bufs[2] = {b.template at<T>(p.felem[p.nlev]), b.template at<T>(p.ksbuf)};
      int cur = 0;
      for (int64_t s = 1; s < K; s *= 2, cur ^= 1) {
        ProfScope ps(PK_FILT_TOP, st);
        launch_team<FWS, TU>(k_filt_ks_team<T, D, TU>, K, st, (const T*)bufs[cur], K, s, (int)(2 * s >= K),
                             bufs[cur ^ 1], b.template at<T>(p.fstate[p.nlev]), x0m, x0L);
      }
    } else {
      ProfScope ps(PK_FILT_TOP, st);
      launch_team<FWS, TSX>(k_filt_top_team<T, D, TSX>, 1, st, (const T*)b.template at<T>(p.felem[p.nlev]),
                            p.cnt[p.nlev], x0m, x0L, b.template at<T>(p.fstate[p.nlev]));
    }
    for (int l = p.nlev - 1; l >= 1; --l) {
      ProfScope ps(PK_FILT_DOWN, st);
      if (p.cnt[l + 1] <= wide)
        launch_team<FWS, TSX>(k_filt_down_team<T, D, TSX>, p.cnt[l + 1], st,
                              (const T*)b.template at<T>(p.felem[l]), p.cnt[l], p.Cg,
                              (const T*)b.template at<T>(p.fstate[l + 1]), p.cnt[l + 1],
                              b.template at<T>(p.fstate[l]));
      else
        launch_team<FWS, TU>(k_filt_down_team<T, D, TU>, p.cnt[l + 1], st, (const T*)b.template at<T>(p.felem[l]),
                             p.cnt[l], p.Cg, (const T*)b.template at<T>(p.fstate[l + 1]), p.cnt[l + 1],
                             b.template at<T>(p.fstate[l]));
    }
    {
      ProfScope ps(PK_FILT_L0_DOWN, st);
      if constexpr (kTeamL0) {
        if (sm.ft_stride)
          launch_l0<TS, true, L0KFWs<T, D, DY, true>>(k_filt_l0_down_team<T, D, DY, TS, true>, n1, st, n, p.C0, sm,
                                                      (const T*)b.template at<T>(p.fstate[1]), n1, means, chols,
                                                      b.template at<T>(p.selem), b.template at<double>(p.partials));
        else
          launch_l0<TS, false, L0KFWs<T, D, DY, false>>(k_filt_l0_down_team<T, D, DY, TS, false>, n1, st, n, p.C0,
                                                        sm, (const T*)b.template at<T>(p.fstate[1]), n1, means, chols,
                                                        b.template at<T>(p.selem), b.template at<double>(p.partials));
      }
      else
        k_filt_l0_down<T, D, DY><<<grid_for(n1, kBlock), kBlock, 0, st>>>(
            n, p.C0, sm, b.template at<T>(p.fstate[1]), n1, means, chols, b.template at<T>(p.selem),
            b.template at<double>(p.partials));
    }
    {
      ProfScope ps(PK_FILT_FINALIZE, st);
      k_finalize_filter<T><<<1, 256, 0, st>>>(b.template at<double>(p.partials), n1, n, DY,
                                              b.template at<double>(p.scalars), b.template at<T>(p.scale));
    }
  }

  // Smoother from the elements left by filter() (or by k_smo_elements) and
  // the terminal state in means/chols[n].
  template <int TS, int TU>
  static void smoother_ts(const Plan& p, char* ws, const T* F, const T* QL, int64_t ft_stride, T* means, T* chols,
                          bool calibrate, const T* means_old, cudaStream_t st) {
    Bufs b{ws, &p};
    const int64_t n = p.n;
    const int64_t n1 = p.cnt[1];
    // one chunk: its end state is the terminal state, written by the top
    // without reading the chunk's composite, which is therefore not built
    if (n1 > 1 || p.ks) {
      ProfScope ps(PK_SMO_L0_REDUCE, st);
      if constexpr (kTeamL0)
        launch_team<SWS, TS>(k_smo_reduce_team<T, D, TS>, n1, st, (const T*)b.template at<T>(p.selem), n, p.C0,
                             b.template at<T>(p.gelem[1]), n1);
      else
        k_smo_reduce<T, D><<<grid_for(n1, kBlock), kBlock, 0, st>>>(b.template at<T>(p.selem), n, p.C0,
                                                                    b.template at<T>(p.gelem[1]), n1);
    }
    const int64_t wide = wide_lane_limit() / TSX;
    for (int l = 1; l < p.nlev; ++l) {
      ProfScope ps(PK_SMO_REDUCE, st);
      if (p.cnt[l + 1] <= wide)
        launch_team<SWS, TSX>(k_smo_reduce_team<T, D, TSX>, p.cnt[l + 1], st,
                              (const T*)b.template at<T>(p.gelem[l]), p.cnt[l], p.Cg,
                              b.template at<T>(p.gelem[l + 1]), p.cnt[l + 1]);
      else
        launch_team<SWS, TU>(k_smo_reduce_team<T, D, TU>, p.cnt[l + 1], st, (const T*)b.template at<T>(p.gelem[l]),
                             p.cnt[l], p.Cg, b.template at<T>(p.gelem[l + 1]), p.cnt[l + 1]);
    }
    if (p.ks) {
      const int64_t K = p.cnt[p.nlev];
      const T* mT = means + n * D;
      const T* LT = chols + n * D * D;
      T* bufs[2] = {b.template at<T>(p.gelem[p.nlev]), b.template at<T>(p.ksbuf)};
      {
        ProfScope ps(PK_SMO_TOP, st);
        launch_team<SWS, TU>(k_smo_abs_team<T, D, TU>, 1, st, bufs[0], K, mT, LT);
      }
      int cur = 0;
      for (int64_t s = 1; s < K; s *= 2, cur ^= 1) {
        ProfScope ps(PK_SMO_TOP, st);
        launch_team<SWS, TU>(k_smo_ks_team<T, D, TU>, K, st, (const T*)bufs[cur], K, s, (int)(2 * s >= K),
                             bufs[cur ^ 1], b.template at<T>(p.gend[p.nlev]), mT, LT);
      }
    } else {
      ProfScope ps(PK_SMO_TOP, st);
      launch_team<SWS, TSX>(k_smo_top_team<T, D, TSX>, 1, st, (const T*)b.template at<T>(p.gelem[p.nlev]),
                            p.cnt[p.nlev], (const T*)(means + n * D), (const T*)(chols + n * D * D),
                            b.template at<T>(p.gend[p.nlev]));
    }
    for (int l = p.nlev - 1; l >= 1; --l) {
      ProfScope ps(PK_SMO_DOWN, st);
      if (p.cnt[l + 1] <= wide)
        launch_team<SWS, TSX>(k_smo_down_team<T, D, TSX>, p.cnt[l + 1], st,
                              (const T*)b.template at<T>(p.gelem[l]), p.cnt[l], p.Cg,
                              (const T*)b.template at<T>(p.gend[l + 1]), p.cnt[l + 1],
                              b.template at<T>(p.gend[l]));
      else
        launch_team<SWS, TU>(k_smo_down_team<T, D, TU>, p.cnt[l + 1], st, (const T*)b.template at<T>(p.gelem[l]),
                             p.cnt[l], p.Cg, (const T*)b.template at<T>(p.gend[l + 1]), p.cnt[l + 1],
                             b.template at<T>(p.gend[l]));
    }
    {
      ProfScope ps(PK_SMO_L0_DOWN, st);
      const T* scl = calibrate ? b.template at<T>(p.scale) : nullptr;
      if constexpr (kTeamL0) {
        if (ft_stride)
          launch_l0<TS, true, SmoL0Ws<T, D, true>>(k_smo_l0_down_team<T, D, TS, true>, n1, st, n, p.C0, F, QL,
                                                   ft_stride, (const T*)b.template at<T>(p.selem),
                                                   (const T*)b.template at<T>(p.gend[1]), n1, means, chols, scl,
                                                   means_old, p.mrtol, p.matol, b.template at<double>(p.partials));
        else
          launch_l0<TS, false, SmoL0Ws<T, D, false>>(k_smo_l0_down_team<T, D, TS, false>, n1, st, n, p.C0, F, QL,
                                                     ft_stride, (const T*)b.template at<T>(p.selem),
                                                     (const T*)b.template at<T>(p.gend[1]), n1, means, chols, scl,
                                                     means_old, p.mrtol, p.matol, b.template at<double>(p.partials));
      }
      else
        k_smo_l0_down<T, D><<<grid_for(n1, kBlock), kBlock, 0, st>>>(
            n, p.C0, F, QL, ft_stride, b.template at<T>(p.selem), b.template at<T>(p.gend[1]), n1, means, chols,
            scl, means_old, p.mrtol, p.matol, b.template at<double>(p.partials));
    }
    {
      ProfScope ps(PK_SMO_FINALIZE, st);
      k_finalize_smoother<<<1, 256, 0, st>>>(b.template at<double>(p.partials), n1,
                                             b.template at<double>(p.scalars));
    }
  }

  static void linearize(int64_t n, int field, const T* params, T p0, T p1, const T* means, T* H, T* c,
                        cudaStream_t st) {
    ProfScope ps(PK_LINEARIZE, st);
    k_linearize<T, D, DY><<<grid_for(n, 128), 128, 0, st>>>(n, field, params, p0, p1, means, H, c);
  }
};

// Smoother elements from given filtered states (used by pof_smoothing, where
// the filtered trajectory comes from the caller).
template <typename T, int D>
__global__ void __launch_bounds__(64) k_smo_elements(int64_t n, const T* __restrict__ F, const T* __restrict__ QL,
                                                     int64_t ft_stride, const T* __restrict__ fmeans,
                                                     const T* __restrict__ fchols, T* __restrict__ selems) {
  using GL = SmoLayout<D>;
  constexpr int D2 = 2 * D;
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n) return;
  const T* Fk = F + k * ft_stride;
  const T* Qk = QL + k * ft_stride;
  const T* m = fmeans + k * D;
  const T* L = fchols + k * D * D;
  T X[D * D2], Y[D * D2];
  mm<T, D, D, D, D, D, D2>(Fk, L, X);
  copy<T, D, D, D, D2>(Qk, X + D);
  copy<T, D, D, D, D2>(L, Y);
  zero<T, D, D, D2>(Y + D);
  tria_top<T, D, D, D2, D2, D2>(X, Y);
  tria<T, D, D, D2>(Y + D);
  T ge[GL::NG];
  T Et[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) Et[i * D + j] = Y[j * D2 + i];
  trsm_lt<T, D, D, D2, D>(X, Et);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) ge[GL::E + i * D + j] = Et[j * D + i];
  T mm_[D], Emp[D];
  mv<T, D, D, D>(Fk, m, mm_);
  mv<T, D, D, D>(ge + GL::E, mm_, Emp);
#pragma unroll
  for (int i = 0; i < D; ++i) ge[GL::G + i] = m[i] - Emp[i];
  copy<T, D, D, D2, D>(Y + D, ge + GL::DM);
  st_soa<T, GL::NG>(selems, n, k, ge);
}

}  // namespace pof
