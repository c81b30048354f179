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

#include <type_traits>

namespace pof {

// ---------------------------------------------------------------------------
// Runtime bounds checks (the sanitizer substitute): compiled in with
// -DPOF_CHECKS (a build with relocatable device code, so every translation
// unit shares one device word), they test the global-memory indices the
// kernels derive from sizes and plan tables -- element, step and problem
// indices -- before the access.  A failing check skips its access and
// records the source line of the first failure in pof_check_line
// (pof_checks_read).  In the normal build every check is the constant true.
// ---------------------------------------------------------------------------
#ifdef POF_CHECKS
extern __device__ unsigned long long pof_check_line;
__device__ __forceinline__ bool pof_check_fail(int line) {
  atomicCAS(&pof_check_line, 0ull, (unsigned long long)line);
  return false;
}
#define POF_IN(i, n) (((i) >= 0 && (i) < (n)) ? true : ::pof::pof_check_fail(__LINE__))
#else
#define POF_IN(i, n) true
#endif

// ---------------------------------------------------------------------------
// Reciprocal and reciprocal square root of a double, for the scalars of the
// Householder reflectors and the diagonal solves.
//
// GB300 runs FP64 at 1/64 of the FP32 rate and a warp instruction holds an
// SM sub-partition's FP64 pipe for the same time however many of its lanes
// are active, so the instruction sequences of IEEE double division and
// square root -- computed once per reflector, often on one lane -- are a
// large share of a small factorization's FP64 instructions.  These take a
// single-precision hardware approximation of the exponent-normalized
// argument as the seed (the float operand and the widened result are built
// with integer operations, so no FP64 conversion is issued), then ONE
// third-order correction in double precision (Householder's iteration of
// order 3; Halley's method for the square root):
//   1/a:       r = 1 - a y,     y <- y (1 + r + r^2)
//   1/sqrt(a): r = 1 - a y^2,   y <- y (1 + r/2 + 3 r^2/8)
// which cubes the seed's relative error (below ~4e-7: truncation of the
// argument to 23 fraction bits plus the approximation) to below 1e-19, so
// the result is within a few units in the last place of the correctly
// rounded value: 3 and 5 FP64 instructions.  Arguments whose binary
// exponent is beyond +-1000 (zero, subnormals, infinities, NaN included)
// take the IEEE operations.
// ---------------------------------------------------------------------------

// double with the sign bit `sign`, binary exponent `e` and the fraction of
// the float f (exact)
__device__ __forceinline__ double widen_with_exp(float f, int e, long long sign) {
  const unsigned fb = __float_as_uint(f);
  const long long ex = (long long)((int)((fb >> 23) & 0xff) - 127 + e + 1023) << 52;
  return __longlong_as_double(sign | ex | ((long long)(fb & 0x7fffff) << 29));
}

__device__ __forceinline__ double rcp_nr(double a) {
  const long long bits = __double_as_longlong(a);
  const int e = (int)((bits >> 52) & 0x7ff) - 1023;
  if (e < -1000 || e > 1000) return 1.0 / a;
  // |a| = m 2^e, m in [1, 2): seed 1/m in single precision, times 2^-e
  const float mf = __int_as_float(0x3f800000 | (int)((bits >> 29) & 0x7fffff));
  const double y = widen_with_exp(__frcp_rn(mf), -e, bits & (1LL << 63));
  const double r = fma(-a, y, 1.0);
  return fma(y, fma(r, r, r), y);
}

__device__ __forceinline__ double rsqrt_nr(double a) {
  const long long bits = __double_as_longlong(a);
  const int e = (int)((bits >> 52) & 0x7ff) - 1023;
  if (e < -1000 || e > 1000 || bits < 0) return 1.0 / sqrt(a);
  // a = m 4^k with m in [1, 4): seed 1/sqrt(m) in single precision, times 2^-k
  const int k = e >> 1;
  const float mf = __int_as_float(((127 + e - 2 * k) << 23) | (int)((bits >> 29) & 0x7fffff));
  const double y = widen_with_exp(rsqrtf(mf), -k, 0);
  const double r = fma(-(a * y), y, 1.0);
  return fma(y, r * fma(r, 0.375, 0.5), y);
}

template <typename T>
__device__ __forceinline__ T rcp(T a) {
  if constexpr (std::is_same<T, double>::value)
    return rcp_nr(a);
  else
    return T(1) / a;
}

// Scalars of the Householder reflector that maps (alpha, x), ||x||^2 = xn2,
// onto (beta, 0), with LAPACK dlarfg's conventions: beta = -sign(alpha)
// ||(alpha, x)|| (sign(0) = +1), tau = (beta - alpha) / beta, the tail
// scaled by scal = 1 / (alpha - beta); no reflection (beta = alpha,
// tau = scal = 0) when x is exactly zero.
template <typename T>
__device__ __forceinline__ void householder(T alpha, T xn2, T& beta, T& tau, T& scal) {
  const bool zero = (xn2 == T(0));
  if constexpr (std::is_same<T, double>::value) {
    const double a2 = fma(alpha, alpha, xn2);
    const double g = rsqrt_nr(a2);  // 1 / ||(alpha, x)||
    // sg = -sign(alpha) g = 1 / beta (sign flipped with an integer operation)
    const double sg = __longlong_as_double(__double_as_longlong(g) ^ (alpha >= 0.0 ? (1LL << 63) : 0LL));
    const double b = a2 * sg;  // beta = -sign(alpha) ||(alpha, x)||
    const double u = alpha - b;
    beta = zero ? alpha : b;
    tau = zero ? 0.0 : -u * sg;  // (beta - alpha) / beta
    scal = zero ? 0.0 : rcp_nr(u);
  } else {
    const T nrm = sqrt(fma(alpha, alpha, xn2));
    beta = zero ? alpha : (alpha >= T(0) ? -nrm : nrm);
    tau = zero ? T(0) : (beta - alpha) / beta;
    scal = zero ? T(0) : T(1) / (alpha - beta);
  }
}

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
    T beta, tau, scal;
    householder(alpha, xn2, beta, tau, scal);
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
    T beta, tau, scal;
    householder(alpha, xn2, beta, tau, scal);
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
    b[i] = s * rcp(L[i * LDL + i]);
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
    b[i] = s * rcp(L[i * LDL + i]);
  }
}

// B(M x NR) <- L^{-1} B
template <typename T, int M, int NR, int LDL, int LDB>
__device__ __forceinline__ void trsm_l(const T* __restrict__ L, T* B) {
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const T inv = rcp(L[i * LDL + i]);
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
    const T inv = rcp(L[i * LDL + i]);
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
