// Per-thread dense linear algebra on small row-major matrices.
//
// Every routine works on one thread's private data with compile-time sizes,
// so loops unroll and index arithmetic folds into immediate offsets.  The
// state dimension D of the solver is small (2..16); at these sizes the FP64
// pipe of a GB300 SM (2 FMA/clk/SM) is the bound, and one thread per chunk of
// time steps keeps every lane of every issued FP64 instruction useful (a
// warp-cooperative Householder leaves most lanes idle on triangular shapes).
//
// Leading dimensions are template parameters so sub-blocks of larger
// matrices (e.g. the two halves of [F L, QL]) are addressed in place.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace pof {

// C(MxN) = A(MxK) * B(KxN)
template <typename T, int M, int K, int N, int LDA, int LDB, int LDC>
__device__ __forceinline__ void mm(const T* __restrict__ A, const T* __restrict__ B, T* __restrict__ C) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < K; ++k) s = fma(A[i * LDA + k], B[k * LDB + j], s);
      C[i * LDC + j] = s;
    }
  }
}

// C(MxN) = A(MxK) * B(KxN) with B lower-triangular (K == N): skips B's zeros.
template <typename T, int M, int K, int LDA, int LDB, int LDC>
__device__ __forceinline__ void mm_lowerB(const T* __restrict__ A, const T* __restrict__ B, T* __restrict__ C) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
#pragma unroll
    for (int j = 0; j < K; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = j; k < K; ++k) s = fma(A[i * LDA + k], B[k * LDB + j], s);
      C[i * LDC + j] = s;
    }
  }
}

// C(MxN) = A^T * B with A (KxM), B (KxN)
template <typename T, int M, int K, int N, int LDA, int LDB, int LDC>
__device__ __forceinline__ void mtm(const T* __restrict__ A, const T* __restrict__ B, T* __restrict__ C) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < K; ++k) s = fma(A[k * LDA + i], B[k * LDB + j], s);
      C[i * LDC + j] = s;
    }
  }
}

// C(MxN) = A(MxK) * B^T with B (NxK)
template <typename T, int M, int K, int N, int LDA, int LDB, int LDC>
__device__ __forceinline__ void mmt(const T* __restrict__ A, const T* __restrict__ B, T* __restrict__ C) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k < K; ++k) s = fma(A[i * LDA + k], B[j * LDB + k], s);
      C[i * LDC + j] = s;
    }
  }
}

// y(M) = A(MxN) x(N)
template <typename T, int M, int N, int LDA>
__device__ __forceinline__ void mv(const T* __restrict__ A, const T* __restrict__ x, T* __restrict__ y) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
    T s = T(0);
#pragma unroll
    for (int k = 0; k < N; ++k) s = fma(A[i * LDA + k], x[k], s);
    y[i] = s;
  }
}

// y(N) = A(MxN)^T x(M)
template <typename T, int M, int N, int LDA>
__device__ __forceinline__ void mtv(const T* __restrict__ A, const T* __restrict__ x, T* __restrict__ y) {
#pragma unroll
  for (int j = 0; j < N; ++j) {
    T s = T(0);
#pragma unroll
    for (int i = 0; i < M; ++i) s = fma(A[i * LDA + j], x[i], s);
    y[j] = s;
  }
}

// In-place lower-triangular square root of an M x NC matrix X (M <= NC):
// on return X[:, :M] holds L (lower triangular) with L L^T = X X^T, and
// X[:, M:] and the strict upper triangle are zero.
//
// This is the LQ factorisation X = L Q computed as LAPACK's dgeqr2 computes
// the R factor of X^T: one Householder reflector per row, in row order, with
// dlarfg's conventions -- beta = -sign(alpha) * ||(alpha, x)||, and no
// reflection (tau = 0, R_jj = alpha) when the tail x is exactly zero.  The
// reference computes tria as qr(A^T, mode="r")^T (pof/utils.py:33-41), so
// the diagonal signs of L match LAPACK's for the same input.
template <typename T, int M, int NC, int LD>
__device__ __forceinline__ void tria(T* X) {
  static_assert(M <= NC, "tria needs M <= NC");
#pragma unroll
  for (int j = 0; j < M; ++j) {
    T* xj = X + j * LD;
    const T alpha = xj[j];
    T xn2 = T(0);
#pragma unroll
    for (int k = j + 1; k < NC; ++k) xn2 = fma(xj[k], xj[k], xn2);
    const bool zero = (xn2 == T(0));
    const T nrm = sqrt(fma(alpha, alpha, xn2));
    const T beta = zero ? alpha : (alpha >= T(0) ? -nrm : nrm);
    const T den = zero ? T(1) : (alpha - beta);
    const T tau = zero ? T(0) : (beta - alpha) / beta;
    const T scal = zero ? T(0) : T(1) / den;
#pragma unroll
    for (int k = j + 1; k < NC; ++k) xj[k] *= scal;  // reflector v (v_j = 1)
    xj[j] = beta;
#pragma unroll
    for (int i = j + 1; i < M; ++i) {
      T* xi = X + i * LD;
      T w = xi[j];
#pragma unroll
      for (int k = j + 1; k < NC; ++k) w = fma(xi[k], xj[k], w);
      w *= tau;
      xi[j] -= w;
#pragma unroll
      for (int k = j + 1; k < NC; ++k) xi[k] = fma(-w, xj[k], xi[k]);
    }
#pragma unroll
    for (int k = j + 1; k < NC; ++k) xj[k] = T(0);
  }
}

// Same reflectors as tria<M, NC>, additionally applied to the MB rows of a
// second block Y (MB x NC, leading dim LDY) that sits below X.  Equivalent to
// the first M reflectors of tria on the stacked (M+MB) x NC matrix [X; Y].
template <typename T, int M, int MB, int NC, int LD, int LDY>
__device__ __forceinline__ void tria_top(T* X, T* Y) {
  static_assert(M <= NC, "tria_top needs M <= NC");
#pragma unroll
  for (int j = 0; j < M; ++j) {
    T* xj = X + j * LD;
    const T alpha = xj[j];
    T xn2 = T(0);
#pragma unroll
    for (int k = j + 1; k < NC; ++k) xn2 = fma(xj[k], xj[k], xn2);
    const bool zero = (xn2 == T(0));
    const T nrm = sqrt(fma(alpha, alpha, xn2));
    const T beta = zero ? alpha : (alpha >= T(0) ? -nrm : nrm);
    const T den = zero ? T(1) : (alpha - beta);
    const T tau = zero ? T(0) : (beta - alpha) / beta;
    const T scal = zero ? T(0) : T(1) / den;
#pragma unroll
    for (int k = j + 1; k < NC; ++k) xj[k] *= scal;
    xj[j] = beta;
#pragma unroll
    for (int i = j + 1; i < M; ++i) {
      T* xi = X + i * LD;
      T w = xi[j];
#pragma unroll
      for (int k = j + 1; k < NC; ++k) w = fma(xi[k], xj[k], w);
      w *= tau;
      xi[j] -= w;
#pragma unroll
      for (int k = j + 1; k < NC; ++k) xi[k] = fma(-w, xj[k], xi[k]);
    }
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      T* yi = Y + i * LDY;
      T w = yi[j];
#pragma unroll
      for (int k = j + 1; k < NC; ++k) w = fma(yi[k], xj[k], w);
      w *= tau;
      yi[j] -= w;
#pragma unroll
      for (int k = j + 1; k < NC; ++k) yi[k] = fma(-w, xj[k], yi[k]);
    }
#pragma unroll
    for (int k = j + 1; k < NC; ++k) xj[k] = T(0);
  }
}

// b <- L^{-1} b   (L lower-triangular M x M)
template <typename T, int M, int LDL>
__device__ __forceinline__ void trsv_l(const T* __restrict__ L, T* b) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
    T s = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) s = fma(-L[i * LDL + k], b[k], s);
    b[i] = s / L[i * LDL + i];
  }
}

// b <- L^{-T} b   (L lower-triangular M x M; back substitution with L^T)
template <typename T, int M, int LDL>
__device__ __forceinline__ void trsv_lt(const T* __restrict__ L, T* b) {
#pragma unroll
  for (int i = M - 1; i >= 0; --i) {
    T s = b[i];
#pragma unroll
    for (int k = i + 1; k < M; ++k) s = fma(-L[k * LDL + i], b[k], s);
    b[i] = s / L[i * LDL + i];
  }
}

// B(M x NR) <- L^{-1} B
template <typename T, int M, int NR, int LDL, int LDB>
__device__ __forceinline__ void trsm_l(const T* __restrict__ L, T* B) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const T inv = T(1) / L[i * LDL + i];
#pragma unroll
    for (int j = 0; j < NR; ++j) {
      T s = B[i * LDB + j];
#pragma unroll
      for (int k = 0; k < i; ++k) s = fma(-L[i * LDL + k], B[k * LDB + j], s);
      B[i * LDB + j] = s * inv;
    }
  }
}

// B(M x NR) <- L^{-T} B
template <typename T, int M, int NR, int LDL, int LDB>
__device__ __forceinline__ void trsm_lt(const T* __restrict__ L, T* B) {
#pragma unroll
  for (int i = M - 1; i >= 0; --i) {
    const T inv = T(1) / L[i * LDL + i];
#pragma unroll
    for (int j = 0; j < NR; ++j) {
      T s = B[i * LDB + j];
#pragma unroll
      for (int k = i + 1; k < M; ++k) s = fma(-L[k * LDL + i], B[k * LDB + j], s);
      B[i * LDB + j] = s * inv;
    }
  }
}

template <typename T, int M, int N, int LDS, int LDD>
__device__ __forceinline__ void copy(const T* __restrict__ S, T* __restrict__ Dst) {
#pragma unroll
  for (int i = 0; i < M; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) Dst[i * LDD + j] = S[i * LDS + j];
}

template <typename T, int M, int N, int LDD>
__device__ __forceinline__ void zero(T* Dst) {
#pragma unroll
  for (int i = 0; i < M; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) Dst[i * LDD + j] = T(0);
}

}  // namespace pof
