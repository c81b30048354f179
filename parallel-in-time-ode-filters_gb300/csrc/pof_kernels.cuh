// Kernels of the chunked three-phase square-root filter and smoother.
//
// Time steps s = 0..n-1 (step s maps grid point s to s+1).  Level-0 chunks
// hold C0 consecutive steps; chunk totals form level 1; levels l >= 1 fold C
// consecutive elements into level l+1 until at most a few remain (the top).
// Every kernel assigns one thread to one chunk.
//
// Internal buffers are structure-of-arrays: field f of element e of a level
// with n elements lives at base[f * n + e], so a warp touching 32
// consecutive elements issues one coalesced access per field.
//
// Caller-facing arrays (x0, F, QL, H, c, R, means, chols) keep the
// reference's row-major layouts: H (n, DY, D), c (n, DY), means (n+1, D),
// chols (n+1, D, D).
#pragma once

#include <stdint.h>

#include "pof_fields.cuh"
#include "pof_ops.cuh"

namespace pof {

struct StepModel {
  const void* F;      // (D, D) or (n, D, D)
  const void* QL;     // (D, D) or (n, D, D)
  int64_t ft_stride;  // elements between consecutive steps' F/QL (0: constant)
  const void* H;      // (n, DY, D)
  const void* c;      // (n, DY)
  const void* R;      // (n, DY, DY), (DY, DY) or nullptr (zero)
  int64_t r_stride;   // elements between consecutive steps' R (0: constant)
};

template <int D>
struct FiltLayout {
  static constexpr int A = 0, B = D * D, U = D * D + D, ETA = 2 * D * D + D, Z = 2 * D * D + 2 * D;
  static constexpr int NF = 3 * D * D + 2 * D;
};
template <int D>
struct SmoLayout {
  static constexpr int G = 0, E = D, DM = D + D * D;
  static constexpr int NG = D + 2 * D * D;
};
template <int D>
struct StateLayout {
  static constexpr int M = 0, L = D;
  static constexpr int NS = D + D * D;
};

// per-chunk partial sums (double accumulators for every T)
enum Partial : int { P_SSQ = 0, P_NLL = 1, P_FOBJ = 2, P_SOBJ = 3, P_NOTCLOSE = 4, P_COUNT = 5 };

template <typename T, int K>
__device__ __forceinline__ void ld_soa(const T* __restrict__ base, int64_t n, int64_t e, T* dst) {
#pragma unroll
  for (int f = 0; f < K; ++f) dst[f] = base[f * n + e];
}
template <typename T, int K>
__device__ __forceinline__ void st_soa(T* __restrict__ base, int64_t n, int64_t e, const T* src) {
#pragma unroll
  for (int f = 0; f < K; ++f) base[f * n + e] = src[f];
}
template <typename T, int K>
__device__ __forceinline__ void ld(const T* __restrict__ src, T* dst) {
#pragma unroll
  for (int f = 0; f < K; ++f) dst[f] = src[f];
}
template <typename T, int K>
__device__ __forceinline__ void st(T* __restrict__ dst, const T* src) {
#pragma unroll
  for (int f = 0; f < K; ++f) dst[f] = src[f];
}

template <typename T, int D, int DY>
struct StepView {
  const T* F;
  const T* QL;
  const T* H;
  const T* c;
  const T* R;
  __device__ __forceinline__ StepView(const StepModel& sm, int64_t s) {
    F = static_cast<const T*>(sm.F) + s * sm.ft_stride;
    QL = static_cast<const T*>(sm.QL) + s * sm.ft_stride;
    H = static_cast<const T*>(sm.H) + s * (DY * D);
    c = static_cast<const T*>(sm.c) + s * DY;
    R = sm.R ? static_cast<const T*>(sm.R) + s * sm.r_stride : nullptr;
  }
};

// ---------------------------------------------------------------------------
// EK1 linearization of a built-in field at means[s+1], s = 0..n-1
// (pof/step.py:12-22 with pof/observations.py:35-40): H = E1 - J(E0 m) E0,
// c = (E1 m - f(E0 m)) - H m, with E0/E1 the Nordsieck-scaled projections
// (pof/convenience.py:26-28): E0 m = p0 * m[i(q+1)], E1 m = p1 * m[i(q+1)+1].
// ---------------------------------------------------------------------------
template <typename T, int D, int DY>
__global__ void k_linearize(int64_t n, int field, const T* __restrict__ params, T p0, T p1,
                            const T* __restrict__ means, T* __restrict__ H, T* __restrict__ c) {
  constexpr int Q1 = D / DY;  // q + 1
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const T* m = means + (s + 1) * D;
  T y[DY], f[DY], J[DY * DY];
#pragma unroll
  for (int i = 0; i < DY; ++i) y[i] = p0 * m[i * Q1];
  field_eval<T, DY>(field, params, y, f, J);
  T h[DY * D];
#pragma unroll
  for (int i = 0; i < DY; ++i) {
#pragma unroll
    for (int k = 0; k < D; ++k) h[i * D + k] = T(0);
#pragma unroll
    for (int j = 0; j < DY; ++j) h[i * D + j * Q1] = -(J[i * DY + j] * p0);
    h[i * D + i * Q1 + 1] += p1;
  }
#pragma unroll
  for (int i = 0; i < DY; ++i) {
    T res = p1 * m[i * Q1 + 1] - f[i];
    T hm = T(0);
#pragma unroll
    for (int k = 0; k < D; ++k) hm = fma(h[i * D + k], m[k], hm);
    c[s * DY + i] = res - hm;
  }
#pragma unroll
  for (int k = 0; k < DY * D; ++k) H[s * DY * D + k] = h[k];
}

// ---------------------------------------------------------------------------
// Filter, phase 1 (level 0): chunk totals.  Chunk 0 runs the filter from x0
// and stores the filtering state as an element with A = 0, eta = 0, Z = 0
// (the operator of filter.py:117-142 reads only b and U of a left operand
// that holds x0).  Other chunks run the conditional fold.
// ---------------------------------------------------------------------------
template <typename T, int D, int DY>
__global__ void __launch_bounds__(64) k_filt_l0_reduce(int64_t n, int C0, StepModel sm, const T* __restrict__ x0m,
                                                       const T* __restrict__ x0L, T* __restrict__ out, int64_t n1) {
  using FL = FiltLayout<D>;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n1) return;
  const int64_t s0 = t * C0;
  const int64_t s1 = (s0 + C0 < n) ? s0 + C0 : n;
  T e[FL::NF];
  if (t == 0) {
    T m[D], L[D * D];
    ld<T, D>(x0m, m);
    ld<T, D * D>(x0L, L);
    T ss, nn;
    {
      StepView<T, D, DY> v(sm, 0);
      kf_step<T, D, DY, false, false>(v.F, v.QL, v.H, v.c, v.R, m, L, ss, nn, nullptr, nullptr, nullptr);
    }
    for (int64_t s = 1; s < s1; ++s) {
      StepView<T, D, DY> v(sm, s);
      kf_step<T, D, DY, false, true>(v.F, v.QL, v.H, v.c, v.R, m, L, ss, nn, nullptr, nullptr, nullptr);
    }
#pragma unroll
    for (int i = 0; i < FL::NF; ++i) e[i] = T(0);
    st<T, D>(e + FL::B, m);
    st<T, D * D>(e + FL::U, L);
  } else {
    T* A = e + FL::A;
    T* b = e + FL::B;
    T* U = e + FL::U;
    T* eta = e + FL::ETA;
    T* Z = e + FL::Z;
#pragma unroll
    for (int i = 0; i < FL::NF; ++i) e[i] = T(0);
#pragma unroll
    for (int i = 0; i < D; ++i) A[i * D + i] = T(1);
    for (int64_t s = s0; s < s1; ++s) {
      if (!POF_IN(s, n)) break;
      StepView<T, D, DY> v(sm, s);
      cond_fold_step<T, D, DY>(v.F, v.QL, v.H, v.c, v.R, A, b, U, eta, Z);
    }
  }
  st_soa<T, FL::NF>(out, n1, t, e);
}

// Filter, phase 2 up-sweep: fold C consecutive general elements.
template <typename T, int D>
__global__ void __launch_bounds__(64) k_filt_reduce(const T* __restrict__ in, int64_t nin, int C, T* __restrict__ out,
                                                    int64_t nout) {
  using FL = FiltLayout<D>;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nout) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < nin) ? i0 + C : nin;
  T a[FL::NF], b[FL::NF];
  ld_soa<T, FL::NF>(in, nin, i0, a);
  for (int64_t i = i0 + 1; i < i1; ++i) {
    ld_soa<T, FL::NF>(in, nin, i, b);
    filt_combine<T, D>(a + FL::A, a + FL::B, a + FL::U, a + FL::ETA, a + FL::Z, b + FL::A, b + FL::B, b + FL::U,
                       b + FL::ETA, b + FL::Z);
  }
  st_soa<T, FL::NF>(out, nout, t, a);
}

// Advance a filtering state over element e (element 0 of every level holds x0
// and is absolute: the state after it is its own (b, U)).
template <typename T, int D>
__device__ __forceinline__ void filt_advance(const T* __restrict__ elems, int64_t n, int64_t i, T* m, T* L) {
  using FL = FiltLayout<D>;
  T e[FL::NF];
  ld_soa<T, FL::NF>(elems, n, i, e);
  if (i == 0) {
    ld<T, D>(e + FL::B, m);
    ld<T, D * D>(e + FL::U, L);
  } else {
    filt_apply<T, D>(m, L, e + FL::A, e + FL::B, e + FL::U, e + FL::ETA, e + FL::Z);
  }
}

// Filter, top of phase 2: the state before each top-level element (one thread).
template <typename T, int D>
__global__ void k_filt_top(const T* __restrict__ elems, int64_t n, const T* __restrict__ x0m,
                           const T* __restrict__ x0L, T* __restrict__ states) {
  using SL = StateLayout<D>;
  if (blockIdx.x * blockDim.x + threadIdx.x != 0) return;
  T st_[SL::NS];
  ld<T, D>(x0m, st_ + SL::M);
  ld<T, D * D>(x0L, st_ + SL::L);
  for (int64_t i = 0; i < n; ++i) {
    st_soa<T, SL::NS>(states, n, i, st_);
    if (i + 1 < n) filt_advance<T, D>(elems, n, i, st_ + SL::M, st_ + SL::L);
  }
}

// Filter, phase 2 down-sweep at level l >= 1: states before every element of
// chunk t from the state before the chunk.
template <typename T, int D>
__global__ void __launch_bounds__(64) k_filt_down(const T* __restrict__ elems, int64_t n, int C,
                                                  const T* __restrict__ states_up, int64_t nup,
                                                  T* __restrict__ states) {
  using SL = StateLayout<D>;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nup) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < n) ? i0 + C : n;
  T st_[SL::NS];
  ld_soa<T, SL::NS>(states_up, nup, t, st_);
  for (int64_t i = i0; i < i1; ++i) {
    st_soa<T, SL::NS>(states, n, i, st_);
    if (i + 1 < i1) filt_advance<T, D>(elems, n, i, st_ + SL::M, st_ + SL::L);
  }
}

// Filter, phase 3 (level 0): the square-root KF inside chunk t from the state
// at its start; writes the filtered states (grid s0+1..s1, and grid 0 for
// chunk 0), the smoother elements of grid points s0..s1-1 and the chunk's
// partial sums (sigma^2, NLL, filter objective).
template <typename T, int D, int DY>
__global__ void __launch_bounds__(64) k_filt_l0_down(int64_t n, int C0, StepModel sm, const T* __restrict__ states1,
                                                     int64_t n1, T* __restrict__ means, T* __restrict__ chols,
                                                     T* __restrict__ selems, double* __restrict__ partials) {
  using SL = StateLayout<D>;
  using GL = SmoLayout<D>;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n1) return;
  const int64_t s0 = t * C0;
  const int64_t s1 = (s0 + C0 < n) ? s0 + C0 : n;
  T st_[SL::NS];
  ld_soa<T, SL::NS>(states1, n1, t, st_);
  T* m = st_ + SL::M;
  T* L = st_ + SL::L;
  if (t == 0) {
    st<T, D>(means, m);
    st<T, D * D>(chols, L);
  }
  double ssq = 0.0, nll = 0.0, fobj = 0.0;
  T ge[GL::NG];
  for (int64_t s = s0; s < s1; ++s) {
    if (!POF_IN(s, n)) break;
    StepView<T, D, DY> v(sm, s);
    T mold[D];
    ld<T, D>(m, mold);
    T ss, nn;
    if (s == 0)
      kf_step<T, D, DY, true, false>(v.F, v.QL, v.H, v.c, v.R, m, L, ss, nn, ge + GL::G, ge + GL::E, ge + GL::DM);
    else
      kf_step<T, D, DY, true, true>(v.F, v.QL, v.H, v.c, v.R, m, L, ss, nn, ge + GL::G, ge + GL::E, ge + GL::DM);
    ssq += (double)ss;
    nll += (double)nn;
    fobj += (double)objective_term<T, D>(v.F, v.QL, mold, m);
    st_soa<T, GL::NG>(selems, n, s, ge);
    st<T, D>(means + (s + 1) * D, m);
    st<T, D * D>(chols + (s + 1) * D * D, L);
  }
  partials[P_SSQ * n1 + t] = ssq;
  partials[P_NLL * n1 + t] = nll;
  partials[P_FOBJ * n1 + t] = fobj;
}

// ---------------------------------------------------------------------------
// Smoother.  Element k (grid point k = 0..n-1) maps the smoothed state at
// k+1 to the one at k; composites of a range [k0, k1) map the state at k1 to
// the state at k0.
// ---------------------------------------------------------------------------
template <typename T, int D>
__global__ void __launch_bounds__(64) k_smo_reduce(const T* __restrict__ in, int64_t nin, int C, T* __restrict__ out,
                                                   int64_t nout) {
  using GL = SmoLayout<D>;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nout) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < nin) ? i0 + C : nin;
  T a[GL::NG], b[GL::NG];
  ld_soa<T, GL::NG>(in, nin, i0, a);
  for (int64_t i = i0 + 1; i < i1; ++i) {
    ld_soa<T, GL::NG>(in, nin, i, b);
    smooth_combine<T, D>(b + GL::G, b + GL::E, b + GL::DM, a + GL::G, a + GL::E, a + GL::DM);
  }
  st_soa<T, GL::NG>(out, nout, t, a);
}

// Top of the smoother hierarchy: the smoothed state after every top-level
// element, starting from the terminal (filtered) state (one thread).
template <typename T, int D>
__global__ void k_smo_top(const T* __restrict__ elems, int64_t n, const T* __restrict__ mT,
                          const T* __restrict__ LT, T* __restrict__ ends) {
  using SL = StateLayout<D>;
  using GL = SmoLayout<D>;
  if (blockIdx.x * blockDim.x + threadIdx.x != 0) return;
  T st_[SL::NS];
  ld<T, D>(mT, st_ + SL::M);
  ld<T, D * D>(LT, st_ + SL::L);
  for (int64_t i = n - 1; i >= 0; --i) {
    st_soa<T, SL::NS>(ends, n, i, st_);
    if (i > 0) {
      T e[GL::NG];
      ld_soa<T, GL::NG>(elems, n, i, e);
      smooth_apply<T, D>(e + GL::G, e + GL::E, e + GL::DM, st_ + SL::M, st_ + SL::L);
    }
  }
}

template <typename T, int D>
__global__ void __launch_bounds__(64) k_smo_down(const T* __restrict__ elems, int64_t n, int C,
                                                 const T* __restrict__ ends_up, int64_t nup, T* __restrict__ ends) {
  using SL = StateLayout<D>;
  using GL = SmoLayout<D>;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nup) return;
  const int64_t i0 = t * C;
  const int64_t i1 = (i0 + C < n) ? i0 + C : n;
  T st_[SL::NS];
  ld_soa<T, SL::NS>(ends_up, nup, t, st_);
  for (int64_t i = i1 - 1; i >= i0; --i) {
    st_soa<T, SL::NS>(ends, n, i, st_);
    if (i > i0) {
      T e[GL::NG];
      ld_soa<T, GL::NG>(elems, n, i, e);
      smooth_apply<T, D>(e + GL::G, e + GL::E, e + GL::DM, st_ + SL::M, st_ + SL::L);
    }
  }
}

// Smoother, phase 3 (level 0): backward recursion inside chunk t from the
// smoothed state at its end.  Writes smoothed means and chols (chols scaled
// by *scale when scale != nullptr), and partial sums of the smoother
// objective and of the convergence test against means_old.
template <typename T, int D>
__global__ void __launch_bounds__(64) k_smo_l0_down(int64_t n, int C0, const T* __restrict__ F,
                                                    const T* __restrict__ QL, int64_t ft_stride,
                                                    const T* __restrict__ selems, const T* __restrict__ ends1,
                                                    int64_t n1, T* __restrict__ means, T* __restrict__ chols,
                                                    const T* __restrict__ scale, const T* __restrict__ means_old,
                                                    double c_mrtol, double c_matol, double* __restrict__ partials) {
  using SL = StateLayout<D>;
  using GL = SmoLayout<D>;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n1) return;
  const int64_t s0 = t * C0;
  const int64_t s1 = (s0 + C0 < n) ? s0 + C0 : n;
  const T sc = scale ? *scale : T(1);
  T st_[SL::NS];
  ld_soa<T, SL::NS>(ends1, n1, t, st_);
  T* m = st_ + SL::M;
  T* L = st_ + SL::L;
  double sobj = 0.0, notclose = 0.0;
  auto close_count = [&](int64_t k, const T* mk) {
    if (!means_old) return;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      const double a = (double)means_old[k * D + i], b = (double)mk[i];
      bool ok;
      if (isfinite(a) && isfinite(b))
        ok = fabs(a - b) <= c_matol + c_mrtol * fabs(b);
      else
        ok = (a == b);
      notclose += ok ? 0.0 : 1.0;
    }
  };
  if (s1 == n) {  // the terminal grid point n belongs to the last chunk
    close_count(n, m);
    if (scale) {
#pragma unroll
      for (int i = 0; i < D * D; ++i) chols[n * D * D + i] = L[i] * sc;
    }
  }
  T ge[GL::NG];
  for (int64_t k = s1 - 1; k >= s0; --k) {
    if (!POF_IN(k, n)) break;
    T mnext[D];
    ld<T, D>(m, mnext);
    ld_soa<T, GL::NG>(selems, n, k, ge);
    smooth_apply<T, D>(ge + GL::G, ge + GL::E, ge + GL::DM, m, L);
    sobj += (double)objective_term<T, D>(F + k * ft_stride, QL + k * ft_stride, m, mnext);
    close_count(k, m);
    st<T, D>(means + k * D, m);
#pragma unroll
    for (int i = 0; i < D * D; ++i) chols[k * D * D + i] = L[i] * sc;
  }
  partials[P_SOBJ * n1 + t] = sobj;
  partials[P_NOTCLOSE * n1 + t] = notclose;
}

// Fixed-order sum of per-chunk partials (deterministic: the same sums in the
// same order on every run).  One block of 256 threads: thread j sums chunks
// j, j+256, ... in order, then a fixed pairwise tree.
template <int NT>
__device__ __forceinline__ double block_sum_fixed(const double* __restrict__ v, int64_t n) {
  __shared__ double red[NT];
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += NT) s += v[i];
  red[threadIdx.x] = s;
  __syncthreads();
#pragma unroll
  for (int w = NT / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

}  // namespace pof
