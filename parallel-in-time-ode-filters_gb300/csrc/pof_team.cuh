// Team-cooperative small-matrix operations: a team of TS lanes of one warp
// (TS = 8, 16 or 32) works on one element combine, matrices in shared
// memory, one matrix row per lane where rows are independent.
//
// Used where there are too few independent combines to give every lane its
// own (the levels >= 1 of the chunked scan, and the single-team top): on a
// GB300 SM a warp instruction occupies the FP64 pipe for ~64 cycles however
// few lanes are active, so a combine spread over TS lanes finishes up to TS
// times sooner than one run by a single lane.
//
// Independent operations of the same shape inside a combine (the two
// triangularizations U and Z, the two triangular solves M and Mu of the
// filter operator) run side by side on the two halves of the team: one
// instruction stream, different operands, half the FP64 instructions.
//
// Layout: row-major with an odd leading dimension (LD = cols + 1 for even
// cols) so the lanes of a team reading one column hit distinct banks.
#pragma once

#include "pof_linalg.cuh"

namespace pof {

template <int TS>
struct Team {
  unsigned mask;
  int r;  // lane index inside the team
  __device__ __forceinline__ Team() {
    const int lane = threadIdx.x & 31;
    r = lane % TS;
    if constexpr (TS == 32)
      mask = 0xffffffffu;
    else
      mask = ((1u << TS) - 1u) << (lane / TS * TS);
  }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  template <typename T>
  __device__ __forceinline__ T sum(T v) const {
#pragma unroll
    for (int o = TS / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, TS);
    return v;
  }
};

// odd leading dimension for a row of `cols` doubles
template <int COLS>
struct Ld {
  static constexpr int v = (COLS % 2 == 0) ? COLS + 1 : COLS;
};

// C(MxN) = op(A) op(B): lanes split the M*N outputs.
// TA: A is stored transposed (K x M, leading dim LDA); TB: B stored as (N x K).
template <typename T, int TS, int M, int K, int N, int LDA, int LDB, int LDC, bool TA = false, bool TB = false>
__device__ __forceinline__ void t_mm(const Team<TS>& tm, const T* A, const T* B, T* C) {
  for (int idx = tm.r; idx < M * N; idx += TS) {
    const int i = idx / N, j = idx % N;
    T s = T(0);
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const T a = TA ? A[k * LDA + i] : A[i * LDA + k];
      const T b = TB ? B[j * LDB + k] : B[k * LDB + j];
      s = fma(a, b, s);
    }
    C[i * LDC + j] = s;
  }
}

// y(M) = op(A) x: lanes split the rows.
template <typename T, int TS, int M, int K, int LDA, bool TA = false>
__device__ __forceinline__ void t_mv(const Team<TS>& tm, const T* A, const T* x, T* y) {
  for (int i = tm.r; i < M; i += TS) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < K; ++k) s = fma(TA ? A[k * LDA + i] : A[i * LDA + k], x[k], s);
    y[i] = s;
  }
}

// In-place tria of an M x NC matrix X (M <= NC) stacked with MB more rows Y
// (Y gets the same reflectors; pass MB = 0 for plain tria).  Same
// reflectors and sign conventions as pof::tria (LAPACK dgeqr2/dlarfg).
// The norm is a team reduction over columns; the row updates run one row per
// lane.  Zeroes X's tails at the end.
//
// wlow > 0 declares X = [X1, X2] with X2 = X[:, wlow:] lower-triangular and
// Y[:, wlow:] zero (the shape of every tria([A, L]) of the filter and
// smoother: [F L, QL], [U1^T Z2, I], [M^T, U2], [E L, D], ...).  Reflector j
// then has no entry beyond column wlow + j (row j of X2 starts with j + 1
// nonzeros and the earlier reflectors only fill columns below wlow + j), so
// its norm, the dot products and the row updates stop there: the same
// arithmetic without the exact zeros.  ncut < NC declares the columns from
// ncut on zero in every row (the observation block [[H Lp, 0], [Lp, 0]] of a
// noiseless update): they stay zero, and the reflectors from ncut - 1 on
// have an empty tail (no reflection: LAPACK's tau = 0, beta = alpha), so
// they are skipped.
//
// A team with at least twice as many lanes as a reflector has rows to update
// (M - 1 + MB) gives each row G = TS / RS lanes (RS: row slots, the next
// power of two): lane phase p takes the columns j + 1 + p, j + 1 + p + G, ...,
// the G partial dot products are summed by shuffles, and each lane updates
// its own columns -- G times fewer FP64 instructions per reflector on the
// latency-bound combines of the upper levels.
template <int R, int TS>
struct RowSlots {
  static constexpr int p2 = R <= 1 ? 1 : (R <= 2 ? 2 : (R <= 4 ? 4 : (R <= 8 ? 8 : (R <= 16 ? 16 : 32))));
  static constexpr int v = p2 < TS ? p2 : TS;
};

template <typename T, int TS, int M, int MB, int NC, int LD, int LDY>
__device__ __forceinline__ void t_tria(const Team<TS>& tm, T* X, T* Y, int wlow = 0, int ncut = NC) {
  constexpr int RS = RowSlots<M - 1 + MB, TS>::v;
  constexpr int G = TS / RS;
  const int src = (threadIdx.x & 31) / TS * TS;  // lane 0 of this team within the warp
  const int mlim = (ncut < NC && ncut - 1 < M) ? ncut - 1 : M;
#pragma unroll 1
  for (int j = 0; j < mlim; ++j) {
    T* xj = X + j * LD;
    int kend = (wlow > 0 && wlow + j + 1 < NC) ? wlow + j + 1 : NC;
    if (ncut < kend) kend = ncut;
    tm.sync();
    // ||x[j, j+1:]||^2: column partials, reduced onto lane 0 (the only one
    // that uses it) over the lanes that hold partials -- the same additions as
    // the full butterfly, without the ones of zeros
    T part = T(0);
    for (int k = j + 1 + tm.r; k < kend; k += TS) part = fma(xj[k], xj[k], part);
    int span = 1;
    while (span < kend - j - 1 && span < TS) span <<= 1;
    for (int o = span >> 1; o > 0; o >>= 1) part += __shfl_xor_sync(tm.mask, part, o, TS);
    const T xn2 = part;
    // the reflector's scalars on one lane (a square root and two divisions
    // are long FP64 sequences), then broadcast
    T tau = T(0), scal = T(0), beta = T(0);
    if (tm.r == 0) householder(xj[j], xn2, beta, tau, scal);
    tau = __shfl_sync(tm.mask, tau, src);
    scal = __shfl_sync(tm.mask, scal, src);
    tm.sync();
    for (int k = j + 1 + tm.r; k < kend; k += TS) xj[k] *= scal;
    if (tm.r == 0) xj[j] = beta;
    tm.sync();
    // rows below j (X rows j+1..M-1, then Y rows 0..MB-1)
    if constexpr (G == 1) {  // one row per lane
      for (int rr = tm.r; rr < (M - j - 1) + MB; rr += TS) {
        T* xi = (rr < M - j - 1) ? X + (j + 1 + rr) * LD : Y + (rr - (M - j - 1)) * LDY;
        T w = xi[j];
        for (int k = j + 1; k < kend; ++k) w = fma(xi[k], xj[k], w);
        w *= tau;
        xi[j] -= w;
        for (int k = j + 1; k < kend; ++k) xi[k] = fma(-w, xj[k], xi[k]);
      }
    } else {  // G lanes per row, column phases; the shuffles need every lane
      const int slot = tm.r % RS, ph = tm.r / RS;
      const int nrows = (M - j - 1) + MB;
      for (int base = 0; base < nrows; base += RS) {
        const int rr = base + slot;
        const bool act = rr < nrows;
        T* xi = act ? ((rr < M - j - 1) ? X + (j + 1 + rr) * LD : Y + (rr - (M - j - 1)) * LDY) : X;
        T part = (act && ph == 0) ? xi[j] : T(0);
        if (act)
          for (int k = j + 1 + ph; k < kend; k += G) part = fma(xi[k], xj[k], part);
#pragma unroll
        for (int o = RS; o < TS; o <<= 1) part += __shfl_xor_sync(tm.mask, part, o, TS);
        if (act) {
          const T w = part * tau;
          if (ph == 0) xi[j] -= w;
          for (int k = j + 1 + ph; k < kend; k += G) xi[k] = fma(-w, xj[k], xi[k]);
        }
      }
    }
  }
  tm.sync();
  for (int idx = tm.r; idx < M * NC; idx += TS) {
    const int i = idx / NC, k = idx % NC;
    if (k > i) X[i * LD + k] = T(0);
  }
  tm.sync();
}

// 1 / L_ii for i = 0..M-1, computed in parallel (lane i) and read by every
// lane through a shuffle: each division is done once per team, not once per
// right-hand side.
template <typename T, int TS, int M, int LDL>
__device__ __forceinline__ T t_recip_diag(const Team<TS>& tm, const T* L) {
  static_assert(M <= TS, "t_recip_diag needs M <= TS");
  return (tm.r < M) ? rcp(L[tm.r * LDL + tm.r]) : T(0);
}

// B(M x NR) <- L^{-1} B (lower L): one right-hand-side column per lane.
template <typename T, int TS, int M, int NR, int LDL, int LDB>
__device__ __forceinline__ void t_trsm_l(const Team<TS>& tm, const T* L, T* B) {
  if constexpr (M <= TS) {
    const int src = (threadIdx.x & 31) / TS * TS;
    const T rd = t_recip_diag<T, TS, M, LDL>(tm, L);
    T rdi[M];
#pragma unroll
    for (int i = 0; i < M; ++i) rdi[i] = __shfl_sync(tm.mask, rd, src + i);
    for (int j = tm.r; j < NR; j += TS) {
#pragma unroll
      for (int i = 0; i < M; ++i) {
        T s = B[i * LDB + j];
#pragma unroll
        for (int k = 0; k < i; ++k) s = fma(-L[i * LDL + k], B[k * LDB + j], s);
        B[i * LDB + j] = s * rdi[i];
      }
    }
  } else {
    for (int j = tm.r; j < NR; j += TS) {
#pragma unroll
      for (int i = 0; i < M; ++i) {
        T s = B[i * LDB + j];
#pragma unroll
        for (int k = 0; k < i; ++k) s = fma(-L[i * LDL + k], B[k * LDB + j], s);
        B[i * LDB + j] = s * rcp(L[i * LDL + i]);
      }
    }
  }
}

// B(M x NR) <- L^{-T} B
template <typename T, int TS, int M, int NR, int LDL, int LDB>
__device__ __forceinline__ void t_trsm_lt(const Team<TS>& tm, const T* L, T* B) {
  if constexpr (M <= TS) {
    const int src = (threadIdx.x & 31) / TS * TS;
    const T rd = t_recip_diag<T, TS, M, LDL>(tm, L);
    T rdi[M];
#pragma unroll
    for (int i = 0; i < M; ++i) rdi[i] = __shfl_sync(tm.mask, rd, src + i);
    for (int j = tm.r; j < NR; j += TS) {
#pragma unroll
      for (int i = M - 1; i >= 0; --i) {
        T s = B[i * LDB + j];
#pragma unroll
        for (int k = i + 1; k < M; ++k) s = fma(-L[k * LDL + i], B[k * LDB + j], s);
        B[i * LDB + j] = s * rdi[i];
      }
    }
  } else {
    for (int j = tm.r; j < NR; j += TS) {
#pragma unroll
      for (int i = M - 1; i >= 0; --i) {
        T s = B[i * LDB + j];
#pragma unroll
        for (int k = i + 1; k < M; ++k) s = fma(-L[k * LDL + i], B[k * LDB + j], s);
        B[i * LDB + j] = s * rcp(L[i * LDL + i]);
      }
    }
  }
}

template <typename T, int TS, int M, int N, int LDS, int LDD, bool TR = false>
__device__ __forceinline__ void t_copy(const Team<TS>& tm, const T* S, T* Dst) {
  for (int idx = tm.r; idx < M * N; idx += TS) {
    const int i = idx / N, j = idx % N;
    Dst[i * LDD + j] = TR ? S[j * LDS + i] : S[i * LDS + j];
  }
}

template <typename T, int TS, int M, int N, int LDD>
__device__ __forceinline__ void t_fill(const Team<TS>& tm, T* Dst, T v, T diag) {
  for (int idx = tm.r; idx < M * N; idx += TS) {
    const int i = idx / N, j = idx % N;
    Dst[i * LDD + j] = (i == j) ? diag : v;
  }
}

// ---------------------------------------------------------------------------
// Element operations (same formulas as pof_ops.cuh, team-parallel)
// ---------------------------------------------------------------------------

// Shared-memory workspace of one team for the filter operations.
template <typename T, int D>
struct FiltTeamWs {
  static constexpr int D2 = 2 * D;
  static constexpr int LD2 = Ld<D2>::v;
  static constexpr int LD1 = Ld<D>::v;
  // element 1 (running) and element 2 (incoming): A, U, Z (D x LD1), b, eta (D)
  T A1[D * LD1], U1[D * LD1], Z1[D * LD1], b1[D], e1[D];
  T A2[D * LD1], U2[D * LD1], Z2[D * LD1], b2[D], e2[D];
  T Xt[D * LD2], Xb[D * LD2];  // [U1^T Z2, I] and [Z2, 0] -> Xi
  T M[D * LD1], Mu[D * LD1], W[D * LD1];
  T UX[D * LD2];
  T v1[D], v2[D], v3[D];
};

// e1 <- e1 (x) e2 (pof/parallel_filtsmooth/filter.py:117-142)
template <typename T, int TS, int D>
__device__ __forceinline__ void t_filt_combine(const Team<TS>& tm, FiltTeamWs<T, D>& w) {
  using W = FiltTeamWs<T, D>;
  constexpr int L1 = W::LD1, L2 = W::LD2, D2 = W::D2;
  // Xi = [[U1^T Z2, I], [Z2, 0]]
  t_mm<T, TS, D, D, D, L1, L1, L2, true, false>(tm, w.U1, w.Z2, w.Xt);
  t_fill<T, TS, D, D, L2>(tm, w.Xt + D, T(0), T(1));
  t_copy<T, TS, D, D, L1, L2>(tm, w.Z2, w.Xb);
  t_fill<T, TS, D, D, L2>(tm, w.Xb + D, T(0), T(0));
  t_tria<T, TS, D, D, D2, L2, L2>(tm, w.Xt, w.Xb, D);   // Xi11 = Xt[:, :D], Xi21 = Xb[:, :D]
  t_tria<T, TS, D, 0, D, L2, L2>(tm, w.Xb + D, w.Xb);  // Xi22 = Xb[:, D:]
  // M = Xi11^{-1} U1^T A2^T ; Mu = Xi11^{-1} U1^T
  t_mm<T, TS, D, D, D, L1, L1, L1, true, true>(tm, w.U1, w.A2, w.M);
  t_copy<T, TS, D, D, L1, L1, true>(tm, w.U1, w.Mu);
  tm.sync();
  {  // M and Mu side by side on the two halves of the team
    const Team<TS / 2> h;
    t_trsm_l<T, TS / 2, D, D, L2, L1>(h, w.Xt, tm.r >= TS / 2 ? w.Mu : w.M);
  }
  tm.sync();
  // W = M^T Xi21^T  ; A_new = (A2 - W) A1  (into UX scratch, then copied)
  t_mm<T, TS, D, D, D, L1, L2, L1, true, true>(tm, w.M, w.Xb, w.W);
  tm.sync();
  for (int idx = tm.r; idx < D * D; idx += TS) {
    const int i = idx / D, j = idx % D;
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(w.A2[i * L1 + k] - w.W[i * L1 + k], w.A1[k * L1 + j], s);
    w.UX[i * L2 + j] = s;
  }
  // b: t2 = b1 + U1 U1^T eta2 ; t3 = Xi21^T t2 ; t2 -= Mu^T t3 ; b = A2 t2 + b2
  t_mv<T, TS, D, D, L1, true>(tm, w.U1, w.e2, w.v1);
  tm.sync();
  t_mv<T, TS, D, D, L1, false>(tm, w.U1, w.v1, w.v2);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.v2[i] += w.b1[i];
  tm.sync();
  t_mv<T, TS, D, D, L2, true>(tm, w.Xb, w.v2, w.v3);
  tm.sync();
  t_mv<T, TS, D, D, L1, true>(tm, w.Mu, w.v3, w.v1);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.v2[i] -= w.v1[i];
  tm.sync();
  t_mv<T, TS, D, D, L1, false>(tm, w.A2, w.v2, w.v3);  // b_new (without b2) in v3
  tm.sync();
  // eta: e = Xi11^{-T} Xi21^T (into Mu) ; t = eta2 - Z2 Z2^T b1 ; t -= e^T U1^T t ; eta = A1^T t + eta1
  t_copy<T, TS, D, D, L2, L1, true>(tm, w.Xb, w.Mu);
  t_mv<T, TS, D, D, L1, true>(tm, w.Z2, w.b1, w.v1);
  tm.sync();
  t_trsm_lt<T, TS, D, D, L2, L1>(tm, w.Xt, w.Mu);
  t_mv<T, TS, D, D, L1, false>(tm, w.Z2, w.v1, w.v2);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.v2[i] = w.e2[i] - w.v2[i];
  for (int i = tm.r; i < D; i += TS) w.b1[i] = w.v3[i] + w.b2[i];  // b1 no longer read
  tm.sync();
  t_mv<T, TS, D, D, L1, true>(tm, w.U1, w.v2, w.v1);
  tm.sync();
  t_mv<T, TS, D, D, L1, true>(tm, w.Mu, w.v1, w.v3);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.v2[i] -= w.v3[i];
  tm.sync();
  t_mv<T, TS, D, D, L1, true>(tm, w.A1, w.v2, w.v3);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.e1[i] = w.v3[i] + w.e1[i];
  // Z = tria([A1^T Xi22, Z1])  (Xt rows reused: A1 is still the old A)
  t_mm<T, TS, D, D, D, L1, L2, L2, true, false>(tm, w.A1, w.Xb + D, w.Xt);
  t_copy<T, TS, D, D, L1, L2>(tm, w.Z1, w.Xt + D);
  tm.sync();
  // A1 <- new A (from UX scratch) ; U = tria([M^T, U2]) in UX
  t_copy<T, TS, D, D, L2, L1>(tm, w.UX, w.A1);
  tm.sync();
  t_copy<T, TS, D, D, L1, L2, true>(tm, w.M, w.UX);
  t_copy<T, TS, D, D, L1, L2>(tm, w.U2, w.UX + D);
  {  // U and Z side by side on the two halves of the team
    const Team<TS / 2> h;
    T* X = tm.r >= TS / 2 ? w.Xt : w.UX;
    t_tria<T, TS / 2, D, 0, D2, L2, L2>(h, X, X, D);
  }
  tm.sync();
  t_copy<T, TS, D, D, L2, L1>(tm, w.UX, w.U1);
  t_copy<T, TS, D, D, L2, L1>(tm, w.Xt, w.Z1);
  tm.sync();
}

// (m, L) <- state after element 2: (b, U) part of the combine with e1 = (m, L)
// held in (b1, U1).
template <typename T, int TS, int D>
__device__ __forceinline__ void t_filt_apply(const Team<TS>& tm, FiltTeamWs<T, D>& w) {
  using W = FiltTeamWs<T, D>;
  constexpr int L1 = W::LD1, L2 = W::LD2, D2 = W::D2;
  t_mm<T, TS, D, D, D, L1, L1, L2, true, false>(tm, w.U1, w.Z2, w.Xt);
  t_fill<T, TS, D, D, L2>(tm, w.Xt + D, T(0), T(1));
  t_copy<T, TS, D, D, L1, L2>(tm, w.Z2, w.Xb);
  t_fill<T, TS, D, D, L2>(tm, w.Xb + D, T(0), T(0));
  t_tria<T, TS, D, D, D2, L2, L2>(tm, w.Xt, w.Xb, D);
  t_mm<T, TS, D, D, D, L1, L1, L1, true, true>(tm, w.U1, w.A2, w.M);
  t_copy<T, TS, D, D, L1, L1, true>(tm, w.U1, w.Mu);
  tm.sync();
  {  // M and Mu side by side on the two halves of the team
    const Team<TS / 2> h;
    t_trsm_l<T, TS / 2, D, D, L2, L1>(h, w.Xt, tm.r >= TS / 2 ? w.Mu : w.M);
  }
  tm.sync();
  t_mv<T, TS, D, D, L1, true>(tm, w.U1, w.e2, w.v1);
  tm.sync();
  t_mv<T, TS, D, D, L1, false>(tm, w.U1, w.v1, w.v2);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.v2[i] += w.b1[i];
  tm.sync();
  t_mv<T, TS, D, D, L2, true>(tm, w.Xb, w.v2, w.v3);
  tm.sync();
  t_mv<T, TS, D, D, L1, true>(tm, w.Mu, w.v3, w.v1);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.v2[i] -= w.v1[i];
  tm.sync();
  t_mv<T, TS, D, D, L1, false>(tm, w.A2, w.v2, w.v3);
  t_copy<T, TS, D, D, L1, L2, true>(tm, w.M, w.UX);
  t_copy<T, TS, D, D, L1, L2>(tm, w.U2, w.UX + D);
  tm.sync();
  for (int i = tm.r; i < D; i += TS) w.b1[i] = w.v3[i] + w.b2[i];
  t_tria<T, TS, D, 0, D2, L2, L2>(tm, w.UX, w.UX, D);
  t_copy<T, TS, D, D, L2, L1>(tm, w.UX, w.U1);
  tm.sync();
}

// Smoother: shared-memory workspace of one team.
template <typename T, int D>
struct SmoTeamWs {
  static constexpr int D2 = 2 * D;
  static constexpr int LD2 = Ld<D2>::v;
  static constexpr int LD1 = Ld<D>::v;
  T E1[D * LD1], D1[D * LD1], g1[D];  // later element (or the state: D1 = L, g1 = m)
  T E2[D * LD1], D2m[D * LD1], g2[D];  // earlier element / running composite
  T X[D * LD2], En[D * LD1];
  T v[D];
};

// composite (g2, E2, D2) <- (g2, E2, D2) o (g1, E1, D1)
// (pof/parallel_filtsmooth/smoother.py:53-63 with elem1 later, elem2 earlier)
template <typename T, int TS, int D>
__device__ __forceinline__ void t_smooth_combine(const Team<TS>& tm, SmoTeamWs<T, D>& w) {
  using W = SmoTeamWs<T, D>;
  constexpr int L1 = W::LD1, L2 = W::LD2, D2 = W::D2;
  t_mv<T, TS, D, D, L1, false>(tm, w.E2, w.g1, w.v);
  t_mm<T, TS, D, D, D, L1, L1, L2>(tm, w.E2, w.D1, w.X);
  t_copy<T, TS, D, D, L1, L2>(tm, w.D2m, w.X + D);
  t_mm<T, TS, D, D, D, L1, L1, L1>(tm, w.E2, w.E1, w.En);
  tm.sync();
  t_tria<T, TS, D, 0, D2, L2, L2>(tm, w.X, w.X, D);
  for (int i = tm.r; i < D; i += TS) w.g2[i] += w.v[i];
  t_copy<T, TS, D, D, L1, L1>(tm, w.En, w.E2);
  t_copy<T, TS, D, D, L2, L1>(tm, w.X, w.D2m);
  tm.sync();
}

// state (g1 = m, D1 = L) <- element (g2, E2, D2) applied: m = E m + g, L = tria([E L, D])
template <typename T, int TS, int D>
__device__ __forceinline__ void t_smooth_apply(const Team<TS>& tm, SmoTeamWs<T, D>& w) {
  using W = SmoTeamWs<T, D>;
  constexpr int L1 = W::LD1, L2 = W::LD2, D2 = W::D2;
  t_mv<T, TS, D, D, L1, false>(tm, w.E2, w.g1, w.v);
  t_mm<T, TS, D, D, D, L1, L1, L2>(tm, w.E2, w.D1, w.X);
  t_copy<T, TS, D, D, L1, L2>(tm, w.D2m, w.X + D);
  tm.sync();
  t_tria<T, TS, D, 0, D2, L2, L2>(tm, w.X, w.X, D);
  for (int i = tm.r; i < D; i += TS) w.g1[i] = w.v[i] + w.g2[i];
  t_copy<T, TS, D, D, L2, L1>(tm, w.X, w.D1);
  tm.sync();
}

}  // namespace pof

namespace pof {

// ---------------------------------------------------------------------------
// Level-0 (per time step) operations, team-parallel.  Same formulas as
// kf_step / cond_fold_step of pof_ops.cuh.
// ---------------------------------------------------------------------------
template <typename T, int D, int DY>
struct StepDims {
  static constexpr int D2 = 2 * D;
  static constexpr int DP = D + DY;
  static constexpr int LD2 = Ld<D2>::v;
  static constexpr int LD1 = Ld<D>::v;
  static constexpr int LDP = Ld<DP>::v;
  static constexpr int LDZ = Ld<D + DY>::v;
};

// Shared-memory workspace of one team for the Kalman filter step fused with
// the smoother element (the transition model F, QL is passed separately:
// one copy per block).
template <typename T, int D, int DY>
struct StepKFWs : StepDims<T, D, DY> {
  using B = StepDims<T, D, DY>;
  T H[DY * B::LD1], c[DY], R[DY * DY];          // observation model of the step
  T m[D], L[D * B::LD1];                        // filtered state
  T X[D * B::LD2], Y[D * B::LD2];               // [F L, QL], [L, 0]
  T P[B::DP * B::LDP];                          // Psi
  T E[D * B::LD1], g[D], mp[D];                 // smoother element, predicted mean
  T sc[4];                                      // scalars: ssq term, nll term
};

// ... for the conditional fold (and the plain Kalman step of a first chunk).
template <typename T, int D, int DY>
struct StepFoldWs : StepDims<T, D, DY> {
  using B = StepDims<T, D, DY>;
  T H[DY * B::LD1], c[DY], R[DY * DY];
  T m[D], L[D * B::LD1];                        // conditional L (or the filtered state)
  T X[D * B::LD2];                              // [F L, QL]
  T P[B::DP * B::LDP];
  T mp[D];
  T A[D * B::LD1], b[D], eta[D], Z[D * B::LD1];  // conditional fold state
  T FA[D * B::LD1], Fb[D], W[DY * B::LD1], w[DY], ZX[D * B::LDZ];
  T sc[4];
};

template <typename T, int TS, int D, int DY, typename WS>
__device__ __forceinline__ void t_load_step(const Team<TS>& tm, WS& w, const T* H, const T* c, const T* R) {
  constexpr int L1 = Ld<D>::v;
  for (int f = tm.r; f < DY * D; f += TS) w.H[(f / D) * L1 + f % D] = H[f];
  for (int f = tm.r; f < DY; f += TS) w.c[f] = c[f];
  for (int f = tm.r; f < DY * DY; f += TS) w.R[f] = R ? R[f] : T(0);
}

// Psi = tria([[H Lp, R], [Lp, 0]]) with Lp = X[:, :D]; then r = H mp + c,
// ssq / nll terms, m <- mp + Psi21 Psi11^{-1} (-r), L <- Psi22.  rzero: R is
// zero (noiseless observation, the EK1 model), so Psi's last DY columns are.
template <typename T, int TS, int D, int DY, bool UPDATE_STATE, typename WS>
__device__ __forceinline__ void t_update(const Team<TS>& tm, WS& w, bool rzero) {
  using W = StepDims<T, D, DY>;
  constexpr int L1 = W::LD1, L2 = W::LD2, LP = W::LDP, DP = W::DP;
  // rows 0..DY-1: [H Lp, R]; rows DY..: [Lp, 0]
  for (int idx = tm.r; idx < DY * D; idx += TS) {
    const int i = idx / D, j = idx % D;
    T s = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(w.H[i * L1 + k], w.X[k * L2 + j], s);
    w.P[i * LP + j] = s;
  }
  for (int idx = tm.r; idx < DY * DY; idx += TS) w.P[(idx / DY) * LP + D + idx % DY] = w.R[idx];
  for (int idx = tm.r; idx < D * DP; idx += TS) {
    const int i = idx / DP, j = idx % DP;
    w.P[(DY + i) * LP + j] = (j < D) ? w.X[i * L2 + j] : T(0);
  }
  tm.sync();
  t_tria<T, TS, DP, 0, DP, LP, LP>(tm, w.P, w.P, 0, rzero ? D : DP);
  if constexpr (UPDATE_STATE) {
    // the DY x DY solves are tiny: every lane does them redundantly
    T r[DY], wv[DY], wq[DY];
#pragma unroll
    for (int i = 0; i < DY; ++i) {
      T s = w.c[i];
#pragma unroll
      for (int k = 0; k < D; ++k) s = fma(w.H[i * L1 + k], w.mp[k], s);
      r[i] = s;
      wv[i] = -s;
      wq[i] = s;
    }
    trsv_l<T, DY, LP>(w.P, wv);
    trsv_lt<T, DY, LP>(w.P, wq);
    T ss = T(0), yy = T(0);
#pragma unroll
    for (int i = 0; i < DY; ++i) {
      ss = fma(wq[i], wq[i], ss);
      yy = fma(wv[i], wv[i], yy);
    }
    // log |Psi11_ii| on lane i (the DY logarithms run side by side)
    const T ld = tm.sum(tm.r < DY ? T(log(fabs(w.P[tm.r * LP + tm.r]))) : T(0));
    if (tm.r == 0) {
      w.sc[0] = ss;
      w.sc[1] = T(0.5) * yy + ld + T(DY) * Log2Pi<T>::half;
    }
    for (int i = tm.r; i < D; i += TS) {
      T acc = w.mp[i];
#pragma unroll
      for (int k = 0; k < DY; ++k) acc = fma(w.P[(DY + i) * LP + k], wv[k], acc);
      w.m[i] = acc;
    }
    t_copy<T, TS, D, D, LP, L1>(tm, w.P + DY * LP + DY, w.L);
    tm.sync();
  }
}

// Zero structure of a step's transition model, found when the model is
// loaded (it is the caller's data: a TransitionModel need not have any).
//   wq: D when QL is lower-triangular (t_tria's wlow for [F L, QL]), else 0;
//   wf: Q when F is block-diagonal with upper-triangular Q x Q blocks (the
//       IWP prior, I_d (x) A_1 with A_1 upper-triangular), else 0;
//   rzero: the observation noise R is zero (noiseless EK1 model).
struct StepStruct {
  int wq, wf;
  bool rzero;
};

// C(D x N) = F B with F's zeros skipped when wf > 0: row i of F has its
// nonzeros in columns i .. (i / wf + 1) wf - 1.  The skipped terms are exact
// zeros, so the result is the dense product's.
template <typename T, int TS, int D, int N, int LDA, int LDB, int LDC>
__device__ __forceinline__ void t_mm_f(const Team<TS>& tm, const T* F, const T* B, T* C, int wf) {
  for (int idx = tm.r; idx < D * N; idx += TS) {
    const int i = idx / N, j = idx % N;
    const int k0 = wf ? i : 0, k1 = wf ? (i / wf + 1) * wf : D;
    T s = T(0);
    for (int k = k0; k < k1; ++k) s = fma(F[i * LDA + k], B[k * LDB + j], s);
    C[i * LDC + j] = s;
  }
}

// y(D) = F x, F's zeros skipped when wf > 0 (as t_mm_f).
template <typename T, int TS, int D, int LDA>
__device__ __forceinline__ void t_mv_f(const Team<TS>& tm, const T* F, const T* x, T* y, int wf) {
  for (int i = tm.r; i < D; i += TS) {
    const int k0 = wf ? i : 0, k1 = wf ? (i / wf + 1) * wf : D;
    T s = T(0);
    for (int k = k0; k < k1; ++k) s = fma(F[i * LDA + k], x[k], s);
    y[i] = s;
  }
}

// One square-root KF step from the filtered state (m, L) at grid s, fused with
// the smoother element (g, E, Dm = Y[:, D:]) of grid s when SMOOTH.  F and
// QL (D x D, leading dimension Ld<D>) are the step's transition model, ss
// its zero structure.
template <typename T, int TS, int D, int DY, bool SMOOTH, typename WS>
__device__ __forceinline__ void t_kf_step(const Team<TS>& tm, WS& w, const T* F, const T* QL, StepStruct ss) {
  using W = StepDims<T, D, DY>;
  constexpr int L1 = W::LD1, L2 = W::LD2, D2 = W::D2;
  const int wq = ss.wq;
  const bool rzero = ss.rzero;
  t_mm_f<T, TS, D, D, L1, L1, L2>(tm, F, w.L, w.X, ss.wf);
  t_copy<T, TS, D, D, L1, L2>(tm, QL, w.X + D);
  t_mv_f<T, TS, D, L1>(tm, F, w.m, w.mp, ss.wf);
  if constexpr (SMOOTH) {
    t_copy<T, TS, D, D, L1, L2>(tm, w.L, w.Y);
    t_fill<T, TS, D, D, L2>(tm, w.Y + D, T(0), T(0));
    tm.sync();
    t_tria<T, TS, D, D, D2, L2, L2>(tm, w.X, w.Y, wq);  // Phi11, Phi21
    t_tria<T, TS, D, 0, D, L2, L2>(tm, w.Y + D, w.Y);  // Phi22
    // E^T = Phi11^{-T} Phi21^T  (E stored transposed in w.E, fixed below)
    t_copy<T, TS, D, D, L2, L1, true>(tm, w.Y, w.E);
    tm.sync();
    t_trsm_lt<T, TS, D, D, L2, L1>(tm, w.X, w.E);
    tm.sync();
    // g = m - E mp = m - (E^T)^T mp
    t_mv<T, TS, D, D, L1, true>(tm, w.E, w.mp, w.g);
    tm.sync();
    for (int i = tm.r; i < D; i += TS) w.g[i] = w.m[i] - w.g[i];
  } else {
    tm.sync();
    t_tria<T, TS, D, 0, D2, L2, L2>(tm, w.X, w.X, wq);
  }
  t_update<T, TS, D, DY, true>(tm, w, rzero);
}

// One step of the conditional fold (cond_fold_step of pof_ops.cuh).
template <typename T, int TS, int D, int DY>
__device__ __forceinline__ void t_cond_fold_step(const Team<TS>& tm, StepFoldWs<T, D, DY>& w, const T* F,
                                                 const T* QL, StepStruct ss) {
  using W = StepDims<T, D, DY>;
  constexpr int L1 = W::LD1, L2 = W::LD2, LP = W::LDP, LZ = W::LDZ, D2 = W::D2;
  const int wq = ss.wq;
  const bool rzero = ss.rzero;
  t_mm_f<T, TS, D, D, L1, L1, L2>(tm, F, w.L, w.X, ss.wf);
  t_copy<T, TS, D, D, L1, L2>(tm, QL, w.X + D);
  t_mm_f<T, TS, D, D, L1, L1, L1>(tm, F, w.A, w.FA, ss.wf);
  t_mv_f<T, TS, D, L1>(tm, F, w.b, w.Fb, ss.wf);
  tm.sync();
  t_tria<T, TS, D, 0, D2, L2, L2>(tm, w.X, w.X, wq);
  t_update<T, TS, D, DY, false>(tm, w, rzero);
  // W = H FA (DY x D), w = H Fb + c, then Psi11^{-1} on both
  t_mm<T, TS, DY, D, D, L1, L1, L1>(tm, w.H, w.FA, w.W);
  for (int i = tm.r; i < DY; i += TS) {
    T s = w.c[i];
#pragma unroll
    for (int k = 0; k < D; ++k) s = fma(w.H[i * L1 + k], w.Fb[k], s);
    w.w[i] = s;
  }
  tm.sync();
  t_trsm_l<T, TS, DY, D, LP, L1>(tm, w.P, w.W);
  tm.sync();
  if (tm.r == 0) trsv_l<T, DY, LP>(w.P, w.w);
  tm.sync();
  // A = FA - Psi21 W ; b = Fb - Psi21 w ; eta -= W^T w ; ZX = [Z, W^T]
  for (int idx = tm.r; idx < D * D; idx += TS) {
    const int i = idx / D, j = idx % D;
    T acc = w.FA[i * L1 + j];
#pragma unroll
    for (int k = 0; k < DY; ++k) acc = fma(-w.P[(DY + i) * LP + k], w.W[k * L1 + j], acc);
    w.A[i * L1 + j] = acc;
  }
  for (int i = tm.r; i < D; i += TS) {
    T acc = w.Fb[i];
#pragma unroll
    for (int k = 0; k < DY; ++k) acc = fma(-w.P[(DY + i) * LP + k], w.w[k], acc);
    w.b[i] = acc;
    T e = w.eta[i];
#pragma unroll
    for (int k = 0; k < DY; ++k) e = fma(-w.W[k * L1 + i], w.w[k], e);
    w.eta[i] = e;
  }
  for (int idx = tm.r; idx < D * (D + DY); idx += TS) {
    const int i = idx / (D + DY), j = idx % (D + DY);
    w.ZX[i * LZ + j] = (j < D) ? w.Z[i * L1 + j] : w.W[(j - D) * L1 + i];
  }
  t_copy<T, TS, D, D, LP, L1>(tm, w.P + DY * LP + DY, w.L);
  tm.sync();
  t_tria<T, TS, D, 0, D + DY, LZ, LZ>(tm, w.ZX, w.ZX);
  t_copy<T, TS, D, D, LZ, L1>(tm, w.ZX, w.Z);
  tm.sync();
}

}  // namespace pof
