// Sequential square-root filter and smoother (the reference's sequential
// twin, pof/sequential_filtsmooth/*): one thread runs the whole trajectory
// of one problem, step after step.  Used for solve(sequential=True) (sIEKS)
// and sequential_eks_solve (EKF + RTS).
#pragma once

#include "pof_kernels.cuh"

namespace pof {

// pof/sequential_filtsmooth/smoother.py:31-48: gain = Phi21 Phi11^{-1},
// m = mf + gain (ms - F mf), L = tria([Phi22, gain Ls]).
template <typename T, int D>
__device__ __forceinline__ void seq_smooth_step(const T* __restrict__ F, const T* __restrict__ QL,
                                                const T* __restrict__ mf, const T* __restrict__ Lf, T* ms, T* Ls) {
  constexpr int D2 = 2 * D;
  T X[D * D2], Y[D * D2];
  mm<T, D, D, D, D, D, D2>(F, Lf, X);
  copy<T, D, D, D, D2>(QL, X + D);
  copy<T, D, D, D, D2>(Lf, Y);
  zero<T, D, D, D2>(Y + D);
  tria_top<T, D, D, D2, D2, D2>(X, Y);
  tria<T, D, D, D2>(Y + D);
  // gain^T = Phi11^{-T} Phi21^T
  T Gt[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) Gt[i * D + j] = Y[j * D2 + i];
  trsm_lt<T, D, D, D2, D>(X, Gt);
  T Fm[D], diff[D];
  mv<T, D, D, D>(F, mf, Fm);
#pragma unroll
  for (int i = 0; i < D; ++i) diff[i] = ms[i] - Fm[i];
  T mn[D];
  mtv<T, D, D, D>(Gt, diff, mn);
#pragma unroll
  for (int i = 0; i < D; ++i) mn[i] += mf[i];
  // [Phi22, gain Ls]
  T Z[D * D2];
  copy<T, D, D, D2, D2>(Y + D, Z);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(Gt[k * D + i], Ls[k * D + j], s);
      Z[i * D2 + D + j] = s;
    }
  tria<T, D, D2, D2>(Z);
  ld<T, D>(mn, ms);
  copy<T, D, D, D2, D>(Z, Ls);
}

// Whole sequential filter (+ smoother when `smooth`) of one trajectory.  FIELD >= 1: EKF,
// linearizing the built-in field at the predicted mean
// (pof/sequential_filtsmooth/filter.py:9-30); FIELD == 0: the linear filter
// with the caller's (H, c, R) (filter.py:33-56).
// scalars[S_NLL] gets +sum log-lik (the sequential twin's sign,
// sequential_filtsmooth/filter.py:23-30), S_SSQ, S_OBJ (smoother).
template <typename T, int D, int DY>
__global__ void k_seq_filtsmooth(int64_t n, StepModel sm, int field, const T* __restrict__ params, T p0, T p1,
                                 const T* __restrict__ x0m, const T* __restrict__ x0L, int smooth,
                                 T* __restrict__ means, T* __restrict__ chols, double* __restrict__ scalars) {
  constexpr int Q1 = D / DY;
  if (blockIdx.x * blockDim.x + threadIdx.x != 0) return;
  T m[D], L[D * D];
  ld<T, D>(x0m, m);
  ld<T, D * D>(x0L, L);
  st<T, D>(means, m);
  st<T, D * D>(chols, L);
  double ssq = 0.0, ell = 0.0;
  for (int64_t s = 0; s < n; ++s) {
    const T* F = static_cast<const T*>(sm.F) + s * sm.ft_stride;
    const T* QL = static_cast<const T*>(sm.QL) + s * sm.ft_stride;
    T Hb[DY * D], cb[DY];
    const T* H;
    const T* c;
    const T* R = nullptr;
    if (field == 0) {
      H = static_cast<const T*>(sm.H) + s * (DY * D);
      c = static_cast<const T*>(sm.c) + s * DY;
      R = sm.R ? static_cast<const T*>(sm.R) + s * sm.r_stride : nullptr;
    } else {
      // EK1 at the predicted mean F m (observations.py:35-40)
      T mp[D];
      mv<T, D, D, D>(F, m, mp);
      T y[DY], f[DY], J[DY * DY];
#pragma unroll
      for (int i = 0; i < DY; ++i) y[i] = p0 * mp[i * Q1];
      field_eval<T, DY>(field, params, y, f, J);
#pragma unroll
      for (int i = 0; i < DY; ++i) {
#pragma unroll
        for (int k = 0; k < D; ++k) Hb[i * D + k] = T(0);
#pragma unroll
        for (int j = 0; j < DY; ++j) Hb[i * D + j * Q1] = -(J[i * DY + j] * p0);
        Hb[i * D + i * Q1 + 1] += p1;
      }
#pragma unroll
      for (int i = 0; i < DY; ++i) {
        T hm = T(0);
#pragma unroll
        for (int k = 0; k < D; ++k) hm = fma(Hb[i * D + k], mp[k], hm);
        cb[i] = (p1 * mp[i * Q1 + 1] - f[i]) - hm;
      }
      H = Hb;
      c = cb;
    }
    T ss, nn;
    if (s == 0)
      kf_step<T, D, DY, false, false>(F, QL, H, c, R, m, L, ss, nn, nullptr, nullptr, nullptr);
    else
      kf_step<T, D, DY, false, true>(F, QL, H, c, R, m, L, ss, nn, nullptr, nullptr, nullptr);
    ssq += (double)ss;
    ell -= (double)nn;
    st<T, D>(means + (s + 1) * D, m);
    st<T, D * D>(chols + (s + 1) * D * D, L);
  }
  // backward pass (pof/sequential_filtsmooth/smoother.py:8-28)
  double obj = 0.0;
  for (int64_t k = n - 1; smooth && k >= 0; --k) {
    const T* F = static_cast<const T*>(sm.F) + k * sm.ft_stride;
    const T* QL = static_cast<const T*>(sm.QL) + k * sm.ft_stride;
    T mf[D], Lf[D * D], mnext[D];
    ld<T, D>(means + k * D, mf);
    ld<T, D * D>(chols + k * D * D, Lf);
    ld<T, D>(m, mnext);
    seq_smooth_step<T, D>(F, QL, mf, Lf, m, L);
    obj += (double)objective_term<T, D>(F, QL, m, mnext);
    st<T, D>(means + k * D, m);
    st<T, D * D>(chols + k * D * D, L);
  }
  scalars[0] = ell;                         // "nll" of the sequential twin (+ log-lik)
  scalars[1] = obj;                         // smoother objective
  scalars[2] = ssq / (double)n / (double)DY;  // sigma^2
}

}  // namespace pof
