// Per-thread operations of the square-root filter/smoother (one time step,
// one element combine), on thread-private arrays.
//
// Notation: D state dimension, DY observation (ODE) dimension, all matrices
// row-major.  Filter elements are (A, b, U, eta, Z) as in
// pof/parallel_filtsmooth/filter.py:50-81; smoother elements (g, E, Dm) as in
// pof/parallel_filtsmooth/smoother.py:37-50.
#pragma once

#include "pof_linalg.cuh"

namespace pof {

template <typename T>
struct Log2Pi {
  static constexpr T half = T(0.91893853320467274178032973640562);  // log(2 pi) / 2
};

// One square-root Kalman filter step (predict with (F, QL), noiseless-style
// update with (H, c, R)) from the filtered state (m, L) at grid point s,
// fused with the smoother element of grid point s.
//
// Phi = tria([[F L, QL], [L, 0]]) (pof/parallel_filtsmooth/smoother.py:42-46);
// its top block is the predicted chol Lp = tria([F L, QL])
// (pof/sequential_filtsmooth/filter.py:59-66) with the same reflectors.
// Psi = tria([[H Lp, R], [Lp, 0]]) (pof/sequential_filtsmooth/filter.py:69-92);
// its top-left block equals the observation chol tria([H Lp, R]) of
// pof/parallel_filtsmooth/filter.py:84-93.
//
// Outputs: m, L <- filtered state at s+1; ssq_term = ||Psi11^{-T} r||^2
// (whiten quirk, pof/utils.py:110-112); nll_term = -log N(r; 0, Psi11 Psi11^T)
// (pof/utils.py:22-30) with r = H F m + c; smoother element (g, E, Dm) of s
// when WANT_SMOOTH.
template <typename T, int D, int DY, bool WANT_SMOOTH, bool L_LOWER = true>
__device__ __forceinline__ void kf_step(const T* __restrict__ F, const T* __restrict__ QL,
                                        const T* __restrict__ H, const T* __restrict__ c,
                                        const T* __restrict__ R, T* m, T* L, T& ssq_term, T& nll_term,
                                        T* g, T* E, T* Dm) {
  constexpr int D2 = 2 * D;
  constexpr int DP = D + DY;
  T X[D * D2];        // [F L, QL]
  T Y[D * D2];        // [L, 0]   (only used when WANT_SMOOTH)
  if constexpr (L_LOWER)
    mm_lowerB<T, D, D, D, D, D2>(F, L, X);
  else
    mm<T, D, D, D, D, D, D2>(F, L, X);  // x0's chol may be any square root
  copy<T, D, D, D, D2>(QL, X + D);
  if constexpr (WANT_SMOOTH) {
    copy<T, D, D, D, D2>(L, Y);
    zero<T, D, D, D2>(Y + D);
    tria_top<T, D, D, D2, D2, D2>(X, Y);  // X[:, :D] = Phi11, Y[:, :D] = Phi21
    tria<T, D, D, D2>(Y + D);             // Y[:, D:] = Phi22
  } else {
    tria<T, D, D2, D2>(X);
  }
  // predicted mean
  T mp[D];
  mv<T, D, D, D>(F, m, mp);
  if constexpr (WANT_SMOOTH) {
    // E = Phi21 Phi11^{-1}  <=>  E^T = Phi11^{-T} Phi21^T
    T Et[D * D];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) Et[i * D + j] = Y[j * D2 + i];
    trsm_lt<T, D, D, D2, D>(X, Et);
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) E[i * D + j] = Et[j * D + i];
    T Emp[D];
    mv<T, D, D, D>(E, mp, Emp);
#pragma unroll
    for (int i = 0; i < D; ++i) g[i] = m[i] - Emp[i];
    copy<T, D, D, D2, D>(Y + D, Dm);
  }
  // update
  T P[DP * DP];
  mm_lowerB<T, DY, D, D, D2, DP>(H, X, P);  // H Lp  (Lp = X[:, :D], lower)
#pragma unroll
  for (int i = 0; i < DY; ++i)
#pragma unroll
    for (int j = 0; j < DY; ++j) P[i * DP + D + j] = R ? R[i * DY + j] : T(0);
  copy<T, D, D, D2, DP>(X, P + DY * DP);
  zero<T, D, DY, DP>(P + DY * DP + D);
  tria<T, DP, DP, DP>(P);
  T r[DY], w[DY], wq[DY];
  mv<T, DY, D, D>(H, mp, r);
#pragma unroll
  for (int i = 0; i < DY; ++i) {
    r[i] += c[i];
    w[i] = -r[i];
    wq[i] = r[i];
  }
  trsv_l<T, DY, DP>(P, w);    // Psi11^{-1} (-r)
  trsv_lt<T, DY, DP>(P, wq);  // Psi11^{-T} r
  T s = T(0), yy = T(0), ld = T(0);
#pragma unroll
  for (int i = 0; i < DY; ++i) {
    s = fma(wq[i], wq[i], s);
    yy = fma(w[i], w[i], yy);
    ld += log(fabs(P[i * DP + i]));
  }
  ssq_term = s;
  nll_term = T(0.5) * yy + ld + T(DY) * Log2Pi<T>::half;
  // m <- mp + Psi21 w ; L <- Psi22
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T acc = mp[i];
#pragma unroll
    for (int k = 0; k < DY; ++k) acc = fma(P[(DY + i) * DP + k], w[k], acc);
    m[i] = acc;
  }
  copy<T, D, D, DP, D>(P + DY * DP + DY, L);
}

// One step of the conditional fold that turns the elements of a chunk into
// their combined element (A, b, U, eta, Z): a Kalman filter conditioned on
// the state x at the chunk start, whose mean is affine in x (A x + b) and
// whose observations carry the information (eta, Z Z^T) about x.  Same
// element as folding pof/parallel_filtsmooth/filter.py:50-81 elements with
// the operator of filter.py:117-142.  Start values: A = I, b = 0, L = 0,
// eta = 0, Z = 0.
template <typename T, int D, int DY>
__device__ __forceinline__ void cond_fold_step(const T* __restrict__ F, const T* __restrict__ QL,
                                               const T* __restrict__ H, const T* __restrict__ c,
                                               const T* __restrict__ R, T* A, T* b, T* L, T* eta,
                                               T* Z) {
  constexpr int D2 = 2 * D;
  constexpr int DP = D + DY;
  constexpr int DZ = D + DY;
  T X[D * D2];
  mm_lowerB<T, D, D, D, D, D2>(F, L, X);
  copy<T, D, D, D, D2>(QL, X + D);
  tria<T, D, D2, D2>(X);  // Lp = X[:, :D]
  T P[DP * DP];
  mm_lowerB<T, DY, D, D, D2, DP>(H, X, P);
#pragma unroll
  for (int i = 0; i < DY; ++i)
#pragma unroll
    for (int j = 0; j < DY; ++j) P[i * DP + D + j] = R ? R[i * DY + j] : T(0);
  copy<T, D, D, D2, DP>(X, P + DY * DP);
  zero<T, D, DY, DP>(P + DY * DP + D);
  tria<T, DP, DP, DP>(P);
  // FA = F A, Fb = F b
  T FA[D * D], Fb[D];
  mm<T, D, D, D, D, D, D>(F, A, FA);
  mv<T, D, D, D>(F, b, Fb);
  // W = Psi11^{-1} H FA (DY x D), w = Psi11^{-1} (H Fb + c)
  T W[DY * D], w[DY];
  mm<T, DY, D, D, D, D, D>(H, FA, W);
  mv<T, DY, D, D>(H, Fb, w);
#pragma unroll
  for (int i = 0; i < DY; ++i) w[i] += c[i];
  trsm_l<T, DY, D, DP, D>(P, W);
  trsv_l<T, DY, DP>(P, w);
  // A = FA - Psi21 W ; b = Fb - Psi21 w ; eta -= W^T w
#pragma unroll
  for (int i = 0; i < D; ++i) {
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T acc = FA[i * D + j];
#pragma unroll
      for (int k = 0; k < DY; ++k) acc = fma(-P[(DY + i) * DP + k], W[k * D + j], acc);
      A[i * D + j] = acc;
    }
    T acc = Fb[i];
#pragma unroll
    for (int k = 0; k < DY; ++k) acc = fma(-P[(DY + i) * DP + k], w[k], acc);
    b[i] = acc;
    T e = eta[i];
#pragma unroll
    for (int k = 0; k < DY; ++k) e = fma(-W[k * D + i], w[k], e);
    eta[i] = e;
  }
  // Z <- tria([Z, W^T])
  T ZX[D * DZ];
  copy<T, D, D, D, DZ>(Z, ZX);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int k = 0; k < DY; ++k) ZX[i * DZ + D + k] = W[k * D + i];
  tria<T, D, DZ, DZ>(ZX);
  copy<T, D, D, DZ, D>(ZX, Z);
  copy<T, D, D, DP, D>(P + DY * DP + DY, L);
}

// The reference combine of two general filter elements,
// pof/parallel_filtsmooth/filter.py:117-142 (e1 earlier, e2 later).
// In-place: (A1, b1, U1, eta1, Z1) <- e1 (x) e2.
template <typename T, int D>
__device__ __forceinline__ void filt_combine(T* A1, T* b1, T* U1, T* eta1, T* Z1, const T* __restrict__ A2,
                                             const T* __restrict__ b2, const T* __restrict__ U2,
                                             const T* __restrict__ eta2, const T* __restrict__ Z2) {
  constexpr int D2 = 2 * D;
  // Xi = [[U1^T Z2, I], [Z2, 0]]
  T Xt[D * D2], Xb[D * D2];
  mtm<T, D, D, D, D, D, D2>(U1, Z2, Xt);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) Xt[i * D2 + D + j] = (i == j) ? T(1) : T(0);
  copy<T, D, D, D, D2>(Z2, Xb);
  zero<T, D, D, D2>(Xb + D);
  tria_top<T, D, D, D2, D2, D2>(Xt, Xb);  // Xi11 = Xt[:, :D], Xi21 = Xb[:, :D]
  tria<T, D, D, D2>(Xb + D);              // Xi22 = Xb[:, D:]
  const T* Xi11 = Xt;
  // M = Xi11^{-1} U1^T A2^T ;  U1^T A2^T = (A2 U1)^T
  T M[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(U1[k * D + i], A2[j * D + k], s);
      M[i * D + j] = s;
    }
  trsm_l<T, D, D, D2, D>(Xi11, M);
  // Mu = Xi11^{-1} U1^T
  T Mu[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) Mu[i * D + j] = U1[j * D + i];
  trsm_l<T, D, D, D2, D>(Xi11, Mu);
  // Xi21^T = (Xb[:, :D])^T ; MX = M^T Xi21^T   (D x D)
  T MX[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(M[k * D + i], Xb[j * D2 + k], s);
      MX[i * D + j] = s;
    }
  // A = A2 A1 - MX A1
  T A[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(A2[i * D + k] - MX[i * D + k], A1[k * D + j], s);
      A[i * D + j] = s;
    }
  // b = A2 (I - Mu^T Xi21^T)(b1 + U1 U1^T eta2) + b2
  T t1[D], t2[D], t3[D];
  mtv<T, D, D, D>(U1, eta2, t1);  // U1^T eta2
  mv<T, D, D, D>(U1, t1, t2);     // U1 U1^T eta2
#pragma unroll
  for (int i = 0; i < D; ++i) t2[i] += b1[i];
  // t3 = Xi21^T t2 ; t1 = Mu^T t3
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(Xb[k * D2 + i], t2[k], s);
    t3[i] = s;
  }
  mtv<T, D, D, D>(Mu, t3, t1);
#pragma unroll
  for (int i = 0; i < D; ++i) t2[i] -= t1[i];
  T bn[D];
  mv<T, D, D, D>(A2, t2, bn);
#pragma unroll
  for (int i = 0; i < D; ++i) bn[i] += b2[i];
  // eta = A1^T (I - e^T U1^T)(eta2 - Z2 Z2^T b1) + eta1 with e = Xi11^{-T} Xi21^T
  T Ee[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) Ee[i * D + j] = Xb[j * D2 + i];
  trsm_lt<T, D, D, D2, D>(Xi11, Ee);
  mtv<T, D, D, D>(Z2, b1, t1);  // Z2^T b1
  mv<T, D, D, D>(Z2, t1, t3);   // Z2 Z2^T b1
#pragma unroll
  for (int i = 0; i < D; ++i) t3[i] = eta2[i] - t3[i];
  mtv<T, D, D, D>(U1, t3, t1);  // U1^T (.)
  mtv<T, D, D, D>(Ee, t1, t2);  // e^T U1^T (.)
#pragma unroll
  for (int i = 0; i < D; ++i) t3[i] -= t2[i];
  T en[D];
  mtv<T, D, D, D>(A1, t3, en);
#pragma unroll
  for (int i = 0; i < D; ++i) en[i] += eta1[i];
  // U = tria([M^T, U2])
  T UX[D * D2];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) UX[i * D2 + j] = M[j * D + i];
  copy<T, D, D, D, D2>(U2, UX + D);
  tria<T, D, D2, D2>(UX);
  // Z = tria([A1^T Xi22, Z1])
  T ZX[D * D2];
  mtm<T, D, D, D, D, D2, D2>(A1, Xb + D, ZX);
  copy<T, D, D, D, D2>(Z1, ZX + D);
  tria<T, D, D2, D2>(ZX);
  // write back
  copy<T, D, D, D, D>(A, A1);
#pragma unroll
  for (int i = 0; i < D; ++i) {
    b1[i] = bn[i];
    eta1[i] = en[i];
  }
  copy<T, D, D, D2, D>(UX, U1);
  copy<T, D, D, D2, D>(ZX, Z1);
}

// (b, U) part of filt_combine with e1 = the filtering state (m, L): the state
// after element e2 (its A1, eta1, Z1 never reach b and U).
template <typename T, int D>
__device__ __forceinline__ void filt_apply(T* m, T* L, const T* __restrict__ A2, const T* __restrict__ b2,
                                           const T* __restrict__ U2, const T* __restrict__ eta2,
                                           const T* __restrict__ Z2) {
  constexpr int D2 = 2 * D;
  T Xt[D * D2], Xb[D * D2];
  mtm<T, D, D, D, D, D, D2>(L, Z2, Xt);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) Xt[i * D2 + D + j] = (i == j) ? T(1) : T(0);
  copy<T, D, D, D, D2>(Z2, Xb);
  zero<T, D, D, D2>(Xb + D);
  tria_top<T, D, D, D2, D2, D2>(Xt, Xb);
  const T* Xi11 = Xt;
  T M[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(L[k * D + i], A2[j * D + k], s);
      M[i * D + j] = s;
    }
  trsm_l<T, D, D, D2, D>(Xi11, M);
  T Mu[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) Mu[i * D + j] = L[j * D + i];
  trsm_l<T, D, D, D2, D>(Xi11, Mu);
  T t1[D], t2[D], t3[D];
  mtv<T, D, D, D>(L, eta2, t1);
  mv<T, D, D, D>(L, t1, t2);
#pragma unroll
  for (int i = 0; i < D; ++i) t2[i] += m[i];
#pragma unroll
  for (int i = 0; i < D; ++i) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(Xb[k * D2 + i], t2[k], s);
    t3[i] = s;
  }
  mtv<T, D, D, D>(Mu, t3, t1);
#pragma unroll
  for (int i = 0; i < D; ++i) t2[i] -= t1[i];
  mv<T, D, D, D>(A2, t2, m);
#pragma unroll
  for (int i = 0; i < D; ++i) m[i] += b2[i];
  T UX[D * D2];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) UX[i * D2 + j] = M[j * D + i];
  copy<T, D, D, D, D2>(U2, UX + D);
  tria<T, D, D2, D2>(UX);
  copy<T, D, D, D2, D>(UX, L);
}

// Smoother composite accumulation, pof/parallel_filtsmooth/smoother.py:53-63
// with elem1 = (g1, E1, D1) later in time and elem2 = the running composite
// (g2, E2, D2) earlier in time.  In place on the composite:
// g2 <- E2 g1 + g2, E2 <- E2 E1, D2 <- tria([E2 D1, D2]).
template <typename T, int D>
__device__ __forceinline__ void smooth_combine(const T* __restrict__ g1, const T* __restrict__ E1,
                                               const T* __restrict__ D1, T* g2, T* E2, T* D2m) {
  constexpr int D2 = 2 * D;
  T gn[D];
  mv<T, D, D, D>(E2, g1, gn);
  T X[D * D2];
  mm_lowerB<T, D, D, D, D, D2>(E2, D1, X);
  copy<T, D, D, D, D2>(D2m, X + D);
  tria<T, D, D2, D2>(X);
  T En[D * D];
  mm<T, D, D, D, D, D, D>(E2, E1, En);
#pragma unroll
  for (int i = 0; i < D; ++i) g2[i] += gn[i];
  copy<T, D, D, D, D>(En, E2);
  copy<T, D, D, D2, D>(X, D2m);
}

// Apply a smoother (composite) element to the smoothed state after it:
// m <- E m + g, L <- tria([E L, Dm]).
template <typename T, int D>
__device__ __forceinline__ void smooth_apply(const T* __restrict__ g, const T* __restrict__ E,
                                             const T* __restrict__ Dm, T* m, T* L) {
  constexpr int D2 = 2 * D;
  T mn[D];
  mv<T, D, D, D>(E, m, mn);
  T X[D * D2];
  mm_lowerB<T, D, D, D, D, D2>(E, L, X);
  copy<T, D, D, D, D2>(Dm, X + D);
  tria<T, D, D2, D2>(X);
#pragma unroll
  for (int i = 0; i < D; ++i) m[i] = mn[i] + g[i];
  copy<T, D, D, D2, D>(X, L);
}

// Objective term of pof/utils.py:97-101 with the reference's swapped
// arguments: || QL^{-1} (m_k - F m_{k+1}) ||^2.
template <typename T, int D>
__device__ __forceinline__ T objective_term(const T* __restrict__ F, const T* __restrict__ QL,
                                            const T* __restrict__ mk, const T* __restrict__ mk1) {
  T r[D];
  mv<T, D, D, D>(F, mk1, r);
#pragma unroll
  for (int i = 0; i < D; ++i) r[i] = mk[i] - r[i];
  trsv_l<T, D, D>(QL, r);
  T s = T(0);
#pragma unroll
  for (int i = 0; i < D; ++i) s = fma(r[i], r[i], s);
  return s;
}

}  // namespace pof
