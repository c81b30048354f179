// The filter and smoother for large state dimensions (D >= 32), on the
// batched dense primitives of pof_dense.cuh.
//
// Same chunked schedule as the small-D kernels' batched form (restated in
// NumPy as oracle.blocked.linear_filtsmooth_blocked(segmented=True) with one
// group at the top): the n steps are cut into P chunks of C0 steps.
//   filter phase 1: every chunk folds its steps into one element
//     (A, b, U, eta, Z) by the conditional fold (the Kalman filter of the
//     chunk conditioned on the state at its start), all chunks at once, one
//     step after the other;
//   filter phase 2: from x0, the state at every chunk start follows by
//     applying the (b, U) part of the reference's sqrt_filtering_operator
//     (pof/parallel_filtsmooth/filter.py:117-142) chunk total after chunk
//     total;
//   filter phase 3: every chunk runs the square-root Kalman filter from its
//     start state (all chunks at once), emitting the filtered marginals and
//     the NLL / sigma^2 terms (filter.py:84-114);
//   smoother: the elements (g, E, D) of every step (smoother.py:37-50) in
//     slabs of steps, each chunk's composite by sqrt_smoothing_operator
//     (smoother.py:53-63), the smoothed state at every chunk end from the
//     terminal state, then every chunk's backward recursion.
// Each step of a phase is a handful of batched launches over the chunks
// (GEMMs, trias, triangular solves), so a launch carries P independent
// D x D problems.
#include <cuda_runtime.h>
#include <stdlib.h>

#include <algorithm>

#include "../../include/pof.h"
#include "pof_dense.cuh"
#include "pof_dense.h"
#include "pof_dense_sched.h"
#include "pof_fields.cuh"

namespace pof {
int cuda_status(cudaError_t e);
int launch_status();
char* aligned_ws(void* ws);

namespace dense {
namespace {

constexpr int64_t kMaxGridYZ = 65535;
constexpr size_t kPanelSmem = 200 * 1024;

int panel_rows(int n, size_t es) {
  int nb = kMaxPanel;
  while (nb > 1 && size_t(nb) * n * es > kPanelSmem) nb >>= 1;
  return nb;
}

// Panels of at least kClusterMinCols columns in batches of at most
// kClusterMaxBatch matrices are factored by a cluster of kClusterSize CTAs
// (k_tria_panel_cl), each holding a quarter of the columns: that puts idle
// SMs to work in the tree levels above the chunks.  At the chunk loops'
// batches (64-256) every SM already holds a panel, and the cluster's
// barriers only add time (reaction-diffusion at D = 640: float32 4.64 s per
// pass against 4.32 s, float64 10.3 s against 9.2 s for 512 steps).
constexpr int kClusterSize = 4;
constexpr int kClusterMinCols = 256;
constexpr int64_t kClusterMaxBatch = 32;

// ---------------------------------------------------------------------------
// launches
// ---------------------------------------------------------------------------
template <typename T>
struct Ctx {
  cudaStream_t st;
  T *V, *TV, *Y;  // tria scratch, maxbatch entries
  int64_t vbs, ybs;
  int64_t maxbatch;

  void gemm(int64_t batch, int M, int N, int K, T alpha, MV<T> A, MV<T> B, T beta, MV<T> C) {
    if (batch <= 0 || M <= 0 || N <= 0) return;
    // grid.y holds the row tiles (at most 65535): taller products go in row blocks
    constexpr int64_t kRows = kMaxGridYZ * 32;
    if (M > kRows) {
      for (int64_t r0 = 0; r0 < M; r0 += kRows)
        gemm(batch, (int)std::min<int64_t>(kRows, M - r0), N, K, alpha, sub(A, r0, 0), B, beta, sub(C, r0, 0));
      return;
    }
    for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
      const int nb = (int)std::min<int64_t>(kMaxGridYZ, batch - b0);
      if (N <= 16) {
        k_gemm<T, 128, 16, 16, 4, 2><<<dim3(cdiv(N, 16), cdiv(M, 128), nb), 256, 0, st>>>(M, N, K, alpha, A, B,
                                                                                             beta, C, b0);
      } else if (M <= 32) {
        k_gemm<T, 32, 128, 16, 2, 8><<<dim3(cdiv(N, 128), cdiv(M, 32), nb), 256, 0, st>>>(M, N, K, alpha, A, B,
                                                                                            beta, C, b0);
      } else if (tensor_f32()) {
        gemm_tensor(dim3(cdiv(N, 64), cdiv(M, 64), nb), M, N, K, alpha, A, B, beta, C, b0);
      } else {
        k_gemm<T, 64, 64, 16, 4, 4><<<dim3(cdiv(N, 64), cdiv(M, 64), nb), 256, 0, st>>>(M, N, K, alpha, A, B, beta,
                                                                                          C, b0);
      }
    }
  }

  // float32 GEMMs of at least 33 x 17 on the tensor cores (3xTF32) unless
  // POF_DENSE_TF32=0 (read per pass); float64 always on the FP64 pipe.
  bool tf32;
  bool tensor_f32() const { return sizeof(T) == 4 && tf32; }
  // D and, when the transition matrix is block-diagonal with blocks of Q1
  // (checked once per pass), Q1; 0: products with F are GEMMs.
  int D, fq1;

  void fmul(int64_t batch, int K, MV<T> F, MV<T> X, T alpha, T beta, MV<T> Yv) {
    if (batch <= 0 || K <= 0) return;
    if (fq1 <= 0 || F.bs != 0) {
      gemm(batch, D, K, D, alpha, F, X, beta, Yv);
      return;
    }
    const int blocks = (int)std::min<int64_t>(cdiv((int64_t)D * K, 256), 1024);
    for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
      const int nb = (int)std::min<int64_t>(kMaxGridYZ, batch - b0);
      k_blockdiag_mm<T><<<dim3(blocks, nb), 256, 0, st>>>(D, fq1, K, F, X, alpha, beta, Yv, b0);
    }
  }
  void gemm_tensor(dim3 grid, int M, int N, int K, T alpha, MV<T> A, MV<T> B, T beta, MV<T> C, int64_t b0) {
    if constexpr (sizeof(T) == 4)
      k_gemm_tf32x3<<<grid, 128, 0, st>>>(M, N, K, alpha, A, B, beta, C, b0);
  }

  void axpby(int64_t batch, int rows, int cols, T alpha, MV<T> X, T beta, MV<T> Yv) {
    if (batch <= 0 || rows <= 0 || cols <= 0) return;
    const int blocks = (int)std::min<int64_t>(cdiv((int64_t)rows * cols, 256), 256);
    for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
      const int nb = (int)std::min<int64_t>(kMaxGridYZ, batch - b0);
      k_axpby2d<T><<<dim3(blocks, nb), 256, 0, st>>>(rows, cols, alpha, X, beta, Yv, b0);
    }
  }
  void copy(int64_t batch, int rows, int cols, MV<T> X, MV<T> Yv) { axpby(batch, rows, cols, T(1), X, T(0), Yv); }

  void fill(int64_t batch, int rows, int cols, T v, T dv, MV<T> Yv) {
    if (batch <= 0 || rows <= 0 || cols <= 0) return;
    const int blocks = (int)std::min<int64_t>(cdiv((int64_t)rows * cols, 256), 256);
    for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
      const int nb = (int)std::min<int64_t>(kMaxGridYZ, batch - b0);
      k_fill2d<T><<<dim3(blocks, nb), 256, 0, st>>>(rows, cols, v, dv, Yv, b0);
    }
  }

  // In place: W (m x n, n >= m) -> L in its first m columns, zeros elsewhere.
  bool cluster_panels;
  void tria(int64_t batch, int m, int n, MV<T> W) {
    if (batch <= 0) return;
    const bool cl = cluster_panels && n >= kClusterMinCols && batch <= kClusterMaxBatch;
    const int nb = cl ? panel_rows((n + kClusterSize - 1) / kClusterSize, sizeof(T)) : panel_rows(n, sizeof(T));
    for (int i0 = 0; i0 < m; i0 += nb) {
      const int nbb = std::min(nb, m - i0);
      const int np = n - i0;
      for (int64_t b0 = 0; b0 < batch; b0 += maxbatch) {
        const int64_t nbt = std::min<int64_t>(maxbatch, batch - b0);
        MV<T> Wb{W.p + b0 * W.bs, W.rs, W.cs, W.bs};
        if (cl && np >= kClusterMinCols) {
          const size_t smem = size_t(nbb) * ((np + kClusterSize - 1) / kClusterSize) * sizeof(T);
          k_tria_panel_cl<T, kClusterSize><<<(unsigned)(nbt * kClusterSize), 256, smem, st>>>(Wb, i0, nbb, np, V, TV,
                                                                                            vbs, 0);
        } else {
          const size_t smem = size_t(nbb) * np * sizeof(T);
          k_tria_panel<T><<<(unsigned)nbt, 512, smem, st>>>(Wb, i0, nbb, np, V, TV, vbs, 0);
        }
        const int mt = m - i0 - nbb;
        if (mt > 0) {
          MV<T> Wtr = sub(Wb, i0 + nbb, i0);
          MV<T> Vt{V, 1, np, vbs};  // V^T (np x nbb)
          MV<T> Yv{Y, nbb, 1, ybs};
          MV<T> TVv{TV, np, 1, vbs};
          gemm(nbt, mt, nbb, np, T(1), Wtr, Vt, T(0), Yv);
          gemm(nbt, mt, np, nbb, T(-1), Yv, TVv, T(1), Wtr);
        }
      }
    }
  }

  // op(L) X = B in place (B: M x K); L lower, or upper when `upper`.
  void trsm(int64_t batch, int M, int K, MV<T> L, bool upper, MV<T> B) {
    if (batch <= 0 || M <= 0 || K <= 0) return;
    if (K <= 8 && 2 * size_t(M) * sizeof(T) <= 48 * 1024) {
      for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
        const int nb = (int)std::min<int64_t>(kMaxGridYZ, batch - b0);
        k_trsv<T><<<dim3(K, nb), 256, 2 * size_t(M) * sizeof(T), st>>>(M, L, upper, B, b0);
      }
      return;
    }
    auto diag = [&](int r0, int nbr) {
      for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
        const int nb = (int)std::min<int64_t>(kMaxGridYZ, batch - b0);
        k_trsm_diag<T><<<dim3(cdiv(K, 128), nb), 128, 0, st>>>(nbr, sub(L, r0, r0), upper, sub(B, r0, 0), K, b0);
      }
    };
    if (!upper) {
      for (int r0 = 0; r0 < M; r0 += kTrsmBlock) {
        const int nbr = std::min(kTrsmBlock, M - r0);
        if (r0 > 0) gemm(batch, nbr, K, r0, T(-1), sub(L, r0, 0), B, T(1), sub(B, r0, 0));
        diag(r0, nbr);
      }
    } else {
      for (int r0 = ((M - 1) / kTrsmBlock) * kTrsmBlock; r0 >= 0; r0 -= kTrsmBlock) {
        const int nbr = std::min(kTrsmBlock, M - r0);
        const int r1 = r0 + nbr;
        if (r1 < M) gemm(batch, nbr, K, M - r1, T(-1), sub(L, r0, r1), sub(B, r1, 0), T(1), sub(B, r0, 0));
        diag(r0, nbr);
      }
    }
  }
  void step_terms(int64_t batch, int d, MV<T> P11, MV<T> w, MV<T> wq, double* nll, double* ssq, int64_t stride) {
    for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
      const int64_t nb = std::min<int64_t>(kMaxGridYZ, batch - b0);
      k_step_terms<T><<<(unsigned)nb, 128, 0, st>>>(d, P11, w, wq, nll, ssq, stride, b0);
    }
  }
  void sqnorm(int64_t batch, int len, MV<T> x, double* out) {
    for (int64_t b0 = 0; b0 < batch; b0 += kMaxGridYZ) {
      const int64_t nb = std::min<int64_t>(kMaxGridYZ, batch - b0);
      k_sqnorm<T><<<(unsigned)nb, 128, 0, st>>>(len, x, out, b0);
    }
  }
  void scalars(const double* nll, const double* ssq, const double* fobj, const double* sobj, int64_t n, int64_t C0,
               int d, double* out, int which) {
    k_dense_scalars<<<1, 32, 0, st>>>(nll, ssq, fobj, sobj, n, C0, d, out, which);
  }
};


// EK1 linearization of the reaction-diffusion FitzHugh-Nagumo field
// (FIELD_FHN_RD) at means[s+1], one CTA per step, the formula of the small-D
// kernel (pof/step.py:12-22, pof/observations.py:35-40): y = E0 m with
// y_j = p0 m[j (q+1)], H = E1 - J(y) E0, c = (E1 m - f(y)) - H m.  The
// Jacobian has four entries per row (the cell, its two periodic neighbours
// and the other species in the cell); duplicates (two cells) add up.
template <typename T>
__global__ void k_linearize_fhn_rd(int64_t n, int D, int d, const T* __restrict__ prm, T p0, T p1,
                                   const T* __restrict__ means, T* __restrict__ H, T* __restrict__ c) {
  const int64_t s = blockIdx.x;
  const int Q1 = D / d, m = d / 2;
  const T* mm = means + (s + 1) * D;
  T* Hs = H + s * (int64_t)d * D;
  for (int64_t l = threadIdx.x; l < (int64_t)d * D; l += blockDim.x) Hs[l] = T(0);
  __syncthreads();
  const T a = prm[0], b = prm[1], cc = prm[2], kv = prm[3], kw = prm[4];
  for (int i = threadIdx.x; i < d; i += blockDim.x) {
    const bool vrow = i < m;
    const int k = vrow ? i : i - m;
    const int km = (k + m - 1) % m, kp = (k + 1) % m;
    const T v = p0 * mm[(int64_t)k * Q1], w = p0 * mm[(int64_t)(m + k) * Q1];
    int col[4];
    T jac[4];
    T f;
    if (vrow) {
      const T vm = p0 * mm[(int64_t)km * Q1], vp = p0 * mm[(int64_t)kp * Q1];
      f = cc * (v - v * v * v / T(3) + w) + kv * (vm - T(2) * v + vp);
      col[0] = km, jac[0] = kv;
      col[1] = k, jac[1] = cc * (T(1) - v * v) - T(2) * kv;
      col[2] = kp, jac[2] = kv;
      col[3] = m + k, jac[3] = cc;
    } else {
      const T wm = p0 * mm[(int64_t)(m + km) * Q1], wp = p0 * mm[(int64_t)(m + kp) * Q1];
      f = -(v - a + b * w) / cc + kw * (wm - T(2) * w + wp);
      col[0] = k, jac[0] = T(-1) / cc;
      col[1] = m + km, jac[1] = kw;
      col[2] = m + k, jac[2] = -b / cc - T(2) * kw;
      col[3] = m + kp, jac[3] = kw;
    }
    T* row = Hs + (int64_t)i * D;
    for (int e = 0; e < 4; ++e) row[(int64_t)col[e] * Q1] -= jac[e] * p0;
    row[(int64_t)i * Q1 + 1] += p1;
    // H m over the row's non-zeros (y-columns and the row's own E1 column)
    T hm = T(0);
    for (int e = 0; e < 4; ++e) {
      bool first = true;
      for (int e2 = 0; e2 < e; ++e2) first = first && col[e2] != col[e];
      if (first) hm = fma(row[(int64_t)col[e] * Q1], mm[(int64_t)col[e] * Q1], hm);
    }
    hm = fma(row[(int64_t)i * Q1 + 1], mm[(int64_t)i * Q1 + 1], hm);
    c[s * d + i] = (p1 * mm[(int64_t)i * Q1 + 1] - f) - hm;
  }
}

template <typename T>
int run(int which, int64_t n, int D, int d, const void* x0m, const void* x0L, const void* F, const void* QL,
        int64_t fts, const void* H, const void* c, const void* R, int64_t rst, void* om, void* oL, double* osc,
        int chunks, void* ws, size_t wsb, cudaStream_t st) {
  Layout<T> sz = layout<T>(nullptr, which, n, D, d, chunks);
  if (wsb < sz.total) return POF_ERR_WORKSPACE;
  Layout<T> L = layout<T>(aligned_ws(ws), which, n, D, d, chunks);
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k_tria_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kPanelSmem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tria_panel_cl<T, kClusterSize>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)kPanelSmem);
    if (e != cudaSuccess) return cuda_status(e);
    attr_set = true;
  }
  const char* e = getenv("POF_DENSE_TF32");
  const char* ec = getenv("POF_DENSE_CLUSTER");
  Ctx<T> cx{st, L.V, L.TV, L.Y, L.vbs, L.ybs, L.maxbatch, !(e && e[0] == '0'), D, 0, !(ec && ec[0] == '0')};
  // one transition matrix: is it block-diagonal (Q1 = D / d, the IWP prior)?
  if (fts == 0 && d >= 1 && D % d == 0 && D / d < D) {
    const int q1 = D / d;
    cudaError_t ce = cudaMemsetAsync(L.flag, 0, sizeof(unsigned int), st);
    if (ce != cudaSuccess) return cuda_status(ce);
    k_offblock_count<T><<<64, 256, 0, st>>>(D, q1, static_cast<const T*>(F), L.flag);
    unsigned int h = 1;
    ce = cudaMemcpyAsync(&h, L.flag, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_status(ce);
    if (h == 0) cx.fq1 = q1;
  }
  run_schedule<T>(cx, L, which, static_cast<const T*>(x0m), static_cast<const T*>(x0L), static_cast<const T*>(F),
                  static_cast<const T*>(QL), fts, static_cast<const T*>(H), static_cast<const T*>(c),
                  static_cast<const T*>(R), rst, static_cast<T*>(om), static_cast<T*>(oL), osc);
  return launch_status();
}

}  // namespace

int linearize(int dtype, int64_t n, int D, int d, int field, const void* params, double p0, double p1,
              const void* means, void* H, void* c, cudaStream_t st) {
  if (field != FIELD_FHN_RD) return POF_ERR_FIELD;
  if (dtype == POF_F32)
    k_linearize_fhn_rd<float><<<(unsigned)n, 256, 0, st>>>(n, D, d, static_cast<const float*>(params), (float)p0,
                                                           (float)p1, static_cast<const float*>(means),
                                                           static_cast<float*>(H), static_cast<float*>(c));
  else
    k_linearize_fhn_rd<double><<<(unsigned)n, 256, 0, st>>>(n, D, d, static_cast<const double*>(params), p0, p1,
                                                            static_cast<const double*>(means),
                                                            static_cast<double*>(H), static_cast<double*>(c));
  return launch_status();
}

size_t workspace_bytes(int dtype, int which, int64_t n, int D, int d, int chunks) {
  if (n < 1 || D < 1) return 0;
  return dtype == POF_F32 ? layout<float>(nullptr, which, n, D, d, chunks).total
                          : layout<double>(nullptr, which, n, D, d, chunks).total;
}

int filtsmooth(int which, int dtype, int64_t n, int D, int d, const void* x0m, const void* x0L, const void* F,
               const void* QL, int64_t fts, const void* H, const void* c, const void* R, int64_t rst, void* om,
               void* oL, double* osc, int chunks, void* ws, size_t wsb, cudaStream_t st) {
  if (dtype == POF_F32)
    return run<float>(which, n, D, d, x0m, x0L, F, QL, fts, H, c, R, rst, om, oL, osc, chunks, ws, wsb, st);
  return run<double>(which, n, D, d, x0m, x0L, F, QL, fts, H, c, R, rst, om, oL, osc, chunks, ws, wsb, st);
}

}  // namespace dense
}  // namespace pof
