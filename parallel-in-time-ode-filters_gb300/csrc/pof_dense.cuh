// Dense linear algebra for large state dimensions (D >= 32): strided batched
// GEMM, blocked Householder LQ ("tria") and triangular solves, on matrix
// views with arbitrary row/column strides (a transpose is a view, not a
// copy).  Every kernel runs one batch of independent matrices (the chunks of
// the filter/smoother schedule, or the steps of a slab); the filter and
// smoother of pof_dense.cu are written on top of these primitives.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pof_dense_views.h"

namespace pof {
namespace dense {

// ---------------------------------------------------------------------------
// C = alpha * A B + beta * C, A (M x K), B (K x N), C (M x N) views; beta == 0
// does not read C.  One CTA per BM x BN tile of one batch entry; the K loop
// stages BK-deep tiles in shared memory with the loads ordered along
// whichever index is contiguous in memory; each thread accumulates TM x TN
// outputs strided across the tile.
// ---------------------------------------------------------------------------
template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    k_gemm(int M, int N, int K, T alpha, MV<T> A, MV<T> B, T beta, MV<T> C, int64_t b0) {
  constexpr int NT = (BM / TM) * (BN / TN);
  constexpr int TX = BN / TN;
  constexpr int TY = BM / TM;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int t = threadIdx.x;
  const int64_t b = b0 + blockIdx.z;
  const T* __restrict__ Ab = A.p + b * A.bs;
  const T* __restrict__ Bb = B.p + b * B.bs;
  T* Cb = C.p + b * C.bs;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int tx = t % TX, ty = t / TX;
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
  const bool a_kc = A.cs == 1;
  const bool b_nc = B.cs == 1;
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int l = t; l < BM * BK; l += NT) {
      int mm, kk;
      if (a_kc) {
        kk = l % BK;
        mm = l / BK;
      } else {
        mm = l % BM;
        kk = l / BM;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? Ab[gm * A.rs + gk * A.cs] : T(0);
    }
    for (int l = t; l < BK * BN; l += NT) {
      int nn, kk;
      if (b_nc) {
        nn = l % BN;
        kk = l / BN;
      } else {
        kk = l % BK;
        nn = l / BK;
      }
      const int gn = n0 + nn, gk = k0 + kk;
      Bs[kk][nn] = (gn < N && gk < K) ? Bb[gk * B.rs + gn * B.cs] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[TM], bv[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + i * TY];
#pragma unroll
      for (int j = 0; j < TN; ++j) bv[j] = Bs[kk][tx + j * TX];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int gm = m0 + ty + i * TY;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gn = n0 + tx + j * TX;
      if (gn >= N) continue;
      T* c = Cb + gm * C.rs + gn * C.cs;
      *c = beta == T(0) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *c);
    }
  }
}

// ---------------------------------------------------------------------------
// float32 GEMM on the tensor cores with 3xTF32 products: every operand is
// split x = hi + lo with hi = tf32(x) and lo = tf32(x - hi), and
// A B ~ lo_A hi_B + hi_A lo_B + hi_A hi_B accumulated in float32 -- the
// error-compensated TF32 scheme of Ootomo & Yokota ("Recovering single
// precision accuracy from Tensor Cores while surpassing the FP32 theoretical
// peak performance", IJHPCA 2022), float32-level accuracy.  mma.sync
// m16n8k8 TF32 (fragment layouts of the PTX ISA); 64 x 64 tiles, 4 warps
// each owning a 32 x 32 quarter (2 x 4 tiles of 16 x 8), BK = 16 staged in
// shared memory with rows padded to 72 floats so a fragment load touches 32
// distinct banks.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_bits(x);
  lo = tf32_bits(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(128, 4)
    k_gemm_tf32x3(int M, int N, int K, float alpha, MV<float> A, MV<float> B, float beta, MV<float> C, int64_t b0) {
  constexpr int BM = 64, BN = 64, BK = 16, PAD = 8, NT = 128, LPT = BM * BK / NT;  // loads per thread (A and B)
  __shared__ float As[2][BK][BM + PAD];
  __shared__ float Bs[2][BK][BN + PAD];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int g = lane >> 2, tq = lane & 3;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int64_t b = b0 + blockIdx.z;
  const float* __restrict__ Ab = A.p + b * A.bs;
  const float* __restrict__ Bb = B.p + b * B.bs;
  float* Cb = C.p + b * C.bs;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  const bool a_kc = A.cs == 1;
  const bool b_nc = B.cs == 1;
  // the next K tile goes through registers while the current one is on the
  // tensor cores (loads ordered along each view's contiguous index)
  float ra[LPT], rb[LPT];
  auto a_idx = [&](int l, int& mm, int& kk) {
    if (a_kc) {
      kk = l % BK;
      mm = l / BK;
    } else {
      mm = l % BM;
      kk = l / BM;
    }
  };
  auto b_idx = [&](int l, int& nn, int& kk) {
    if (b_nc) {
      nn = l % BN;
      kk = l / BN;
    } else {
      kk = l % BK;
      nn = l / BK;
    }
  };
  auto load = [&](int k0) {
#pragma unroll
    for (int i = 0; i < LPT; ++i) {
      int mm, kk;
      a_idx(t + i * NT, mm, kk);
      const int gm = m0 + mm, gk = k0 + kk;
      ra[i] = (gm < M && gk < K) ? Ab[gm * A.rs + gk * A.cs] : 0.f;
      int nn;
      b_idx(t + i * NT, nn, kk);
      const int gn = n0 + nn, gk2 = k0 + kk;
      rb[i] = (gn < N && gk2 < K) ? Bb[gk2 * B.rs + gn * B.cs] : 0.f;
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int i = 0; i < LPT; ++i) {
      int mm, kk;
      a_idx(t + i * NT, mm, kk);
      As[buf][kk][mm] = ra[i];
      int nn;
      b_idx(t + i * NT, nn, kk);
      Bs[buf][kk][nn] = rb[i];
    }
  };
  load(0);
  store(0);
  __syncthreads();
  for (int k0 = 0, cur = 0; k0 < K; k0 += BK, cur ^= 1) {
    const bool more = k0 + BK < K;
    if (more) load(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; kk += 8) {
      uint32_t ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int mr = wm + i * 16 + g;
        split_tf32(As[cur][kk + tq][mr], ah[i][0], al[i][0]);
        split_tf32(As[cur][kk + tq][mr + 8], ah[i][1], al[i][1]);
        split_tf32(As[cur][kk + tq + 4][mr], ah[i][2], al[i][2]);
        split_tf32(As[cur][kk + tq + 4][mr + 8], ah[i][3], al[i][3]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nc = wn + j * 8 + g;
        split_tf32(Bs[cur][kk + tq][nc], bh[j][0], bl[j][0]);
        split_tf32(Bs[cur][kk + tq + 4][nc], bh[j][1], bl[j][1]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          mma_tf32(acc[i][j], al[i], bh[j]);
          mma_tf32(acc[i][j], ah[i], bl[j]);
          mma_tf32(acc[i][j], ah[i], bh[j]);
        }
    }
    if (more) store(cur ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int gm = m0 + wm + i * 16 + g + (r >= 2 ? 8 : 0);
        const int gn = n0 + wn + j * 8 + 2 * tq + (r & 1);
        if (gm < M && gn < N) {
          float* c = Cb + gm * C.rs + gn * C.cs;
          *c = beta == 0.f ? alpha * acc[i][j][r] : fmaf(alpha, acc[i][j][r], beta * *c);
        }
      }
}

// ---------------------------------------------------------------------------
// Blocked Householder LQ (tria): W (m x n, n >= m) is overwritten so that its
// first m columns hold L (lower triangular, zeros above the diagonal) with
// L L^T = W W^T and columns m..n-1 are zero.  Row reflectors with LAPACK's
// dlarfg convention (beta = -sign(alpha) * ||x||, tau = (beta - alpha) /
// beta, tau = 0 when the tail is zero), the signs numpy.linalg.qr of W^T
// gives.  Panels of nb rows: k_tria_panel factors the panel rows in shared
// memory and writes V (unit upper trapezoidal, nb x n') and T V (the compact
// WY factor applied from the right, H_0 ... H_{nb-1} = I - V^T T V); two
// GEMMs then update the rows below: W_tr <- W_tr - (W_tr V^T)(T V).
// ---------------------------------------------------------------------------
template <typename T>
__device__ inline T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = T(0);
  for (int w = 0; w < nw; ++w) s += red[w];
  return s;
}

template <typename T>
__device__ inline T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One CTA per batch entry.  Dynamic shared memory: nbb * np elements.
// V and TV are nbb x np, row-major, vbs elements apart per batch entry.
// Row r of the panel belongs to warp r mod (warps): that warp applies every
// reflector to it and, right after reflector r - 1, computes the squared
// norm of its tail beyond column r (look-ahead), so each reflector costs one
// block barrier.  A reflector's vector is v = (1, scale * x) with x the
// unscaled tail of its row; products with v fold the scale in, and the
// reflector rows are scaled once at the end.
template <typename T>
__global__ void __launch_bounds__(512)
    k_tria_panel(MV<T> W, int i0, int nbb, int np, T* __restrict__ V, T* __restrict__ TV, int64_t vbs, int64_t b0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);
  __shared__ T nrm[kMaxPanel], scl[kMaxPanel];
  __shared__ T tau[kMaxPanel], beta[kMaxPanel];
  __shared__ T Tm[kMaxPanel][kMaxPanel + 1];
  __shared__ T G[kMaxPanel][kMaxPanel + 1];
  const int t = threadIdx.x, bd = blockDim.x;
  const int lane = t & 31, warp = t >> 5, nw = bd >> 5;
  const int64_t b = b0 + blockIdx.x;
  T* Wb = W.p + b * W.bs + i0 * W.rs + i0 * W.cs;
  for (int l = t; l < nbb * np; l += bd) {
    const int r = l / np, c = l - r * np;
    P[l] = Wb[r * W.rs + c * W.cs];
  }
  __syncthreads();
  if (warp == 0) {  // squared norm of row 0's tail
    T s = T(0);
    for (int c = 1 + lane; c < np; c += 32) s += P[c] * P[c];
    s = warp_sum(s);
    if (lane == 0) nrm[0] = s;
  }
  __syncthreads();
  for (int j = 0; j < nbb; ++j) {
    const T* pr = P + j * np;
    const T alpha = pr[j], s = nrm[j];
    T bj, tj, scale;
    if (s == T(0)) {
      tj = T(0);
      bj = alpha;
      scale = T(0);
    } else {
      const T h = hypot(alpha, sqrt(s));
      bj = alpha >= T(0) ? -h : h;
      tj = (bj - alpha) / bj;
      scale = T(1) / (alpha - bj);
    }
    if (t == 0) {
      tau[j] = tj;
      beta[j] = bj;
      scl[j] = scale;
    }
    // this warp's rows below j: q <- q - tau (q . v) v
    for (int r = warp; r < nbb; r += nw) {
      if (r <= j) continue;
      T* q = P + r * np;
      if (tj != T(0)) {
        T dsum = T(0);
        for (int c = j + 1 + lane; c < np; c += 32) dsum += q[c] * pr[c];
        dsum = warp_sum(dsum);
        const T f = tj * (q[j] + scale * dsum);
        const T fs = f * scale;
        __syncwarp();
        for (int c = j + 1 + lane; c < np; c += 32) q[c] -= fs * pr[c];
        if (lane == 0) q[j] -= f;
        __syncwarp();
      }
      if (r == j + 1) {  // look-ahead: the next reflector's norm
        T s2 = T(0);
        for (int c = j + 2 + lane; c < np; c += 32) s2 += q[c] * q[c];
        s2 = warp_sum(s2);
        if (lane == 0) nrm[j + 1] = s2;
      }
    }
    __syncthreads();
  }
  // panel rows of W: L entries left of the diagonal, beta on it, zeros right
  for (int l = t; l < nbb * np; l += bd) {
    const int r = l / np, c = l - r * np;
    Wb[r * W.rs + c * W.cs] = c < r ? P[l] : (c == r ? beta[r] : T(0));
  }
  __syncthreads();
  // P -> V (unit upper trapezoidal, the tails scaled)
  for (int l = t; l < nbb * np; l += bd) {
    const int r = l / np, c = l - r * np;
    P[l] = c < r ? T(0) : (c == r ? T(1) : P[l] * scl[r]);
  }
  __syncthreads();
  // Gram matrix of the reflectors (upper part)
  for (int pr_ = warp; pr_ < nbb * nbb; pr_ += nw) {
    const int i = pr_ / nbb, j = pr_ - i * nbb;
    if (i >= j) continue;
    T dsum = T(0);
    for (int c = j + lane; c < np; c += 32) dsum += P[i * np + c] * P[j * np + c];
    dsum = warp_sum(dsum);
    if (lane == 0) G[i][j] = dsum;
  }
  __syncthreads();
  // T (upper triangular, forward column recurrence of dlarft)
  if (warp == 0) {
    for (int j = 0; j < nbb; ++j) {
      if (lane < j) {
        T acc = T(0);
        for (int k = lane; k < j; ++k) acc += Tm[lane][k] * G[k][j];
        Tm[lane][j] = -tau[j] * acc;
      }
      if (lane == 0) Tm[j][j] = tau[j];
      if (lane > j && lane < nbb) Tm[lane][j] = T(0);
      __syncwarp();
    }
  }
  __syncthreads();
  T* Vb = V + (int64_t)blockIdx.x * vbs;
  T* TVb = TV + (int64_t)blockIdx.x * vbs;
  for (int c = t; c < np; c += bd) {
    for (int i = 0; i < nbb; ++i) {
      T acc = T(0);
      for (int k = i; k < nbb; ++k) acc = fma(Tm[i][k], P[k * np + c], acc);
      Vb[i * np + c] = P[i * np + c];
      TVb[i * np + c] = acc;
    }
  }
}

// The same panel factorization shared by a thread-block cluster of CS CTAs
// per matrix: CTA r of the cluster holds the panel columns
// [r w, (r + 1) w), w = ceil(np / CS), in its shared memory.  Per reflector
// two cluster-wide reductions through distributed shared memory: the squared
// norm of the row tail (with alpha from the CTA that holds the diagonal
// column), then the dot products of the rows below with the reflector; the
// partial sums are double-buffered by the reflector's parity, so two cluster
// barriers per reflector order every write after the reads of the previous
// use.  Every CTA runs the same sequence of barriers (no early exit).  The
// Gram matrix of the reflectors is reduced the same way; T is formed in
// every CTA (identical inputs, identical order); each CTA writes its columns
// of the panel rows, V and T V.  Results equal k_tria_panel's up to the
// order of the partial sums.
template <typename T, int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(256)
    k_tria_panel_cl(MV<T> W, int i0, int nbb, int np, T* __restrict__ V, T* __restrict__ TV, int64_t vbs,
                    int64_t b0) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* P = reinterpret_cast<T*>(smem_raw);  // nbb x w, row-major
  __shared__ T red[32];
  __shared__ T sq[2], al[2];
  __shared__ T dots[2][kMaxPanel];
  __shared__ T tau[kMaxPanel], beta[kMaxPanel];
  __shared__ T Tm[kMaxPanel][kMaxPanel + 1];
  __shared__ T G[kMaxPanel][kMaxPanel + 1];
  const int t = threadIdx.x, bd = blockDim.x;
  const int lane = t & 31, warp = t >> 5, nw = bd >> 5;
  const int rank = (int)cluster.block_rank();
  const int64_t b = b0 + blockIdx.x / CS;
  const int w = (np + CS - 1) / CS;
  const int c0 = rank * w;
  const int wl = max(0, min(np, c0 + w) - c0);  // columns held here
  T* Wb = W.p + b * W.bs + i0 * W.rs + i0 * W.cs;
  for (int l = t; l < nbb * wl; l += bd) {
    const int r = l / wl, c = l - r * wl;
    P[r * w + c] = Wb[r * W.rs + (c0 + c) * W.cs];
  }
  __syncthreads();
  for (int j = 0; j < nbb; ++j) {
    const int pb = j & 1;
    const int own = j / w;  // rank holding column j
    T* pr = P + j * w;
    // partial squared norm of row j beyond column j
    T s = T(0);
    for (int c = t; c < wl; c += bd)
      if (c0 + c > j) s += pr[c] * pr[c];
    s = block_sum(s, red);
    if (t == 0) {
      sq[pb] = s;
      if (rank == own) al[pb] = pr[j - c0];
    }
    cluster.sync();
    T tot = T(0);
    for (int r = 0; r < CS; ++r) tot += *cluster.map_shared_rank(&sq[pb], r);
    const T alpha = *cluster.map_shared_rank(&al[pb], own);
    T bj, tj, scale;
    if (tot == T(0)) {
      tj = T(0);
      bj = alpha;
      scale = T(0);
    } else {
      const T h = hypot(alpha, sqrt(tot));
      bj = alpha >= T(0) ? -h : h;
      tj = (bj - alpha) / bj;
      scale = T(1) / (alpha - bj);
    }
    for (int c = t; c < wl; c += bd)
      if (c0 + c > j) pr[c] *= scale;
    if (t == 0) {
      if (rank == own) pr[j - c0] = T(1);
      tau[j] = tj;
      beta[j] = bj;
    }
    __syncthreads();
    // partial dot products of the rows below with the reflector
    for (int r = j + 1 + warp; r < nbb; r += nw) {
      const T* q = P + r * w;
      T dsum = T(0);
      for (int c = lane; c < wl; c += 32)
        if (c0 + c >= j) dsum += q[c] * pr[c];
      dsum = warp_sum(dsum);
      if (lane == 0) dots[pb][r] = dsum;
    }
    cluster.sync();
    if (tj != T(0)) {
      for (int r = j + 1 + warp; r < nbb; r += nw) {
        T dsum = T(0);
        if (lane < CS) dsum = *cluster.map_shared_rank(&dots[pb][r], lane);
        dsum = warp_sum(dsum) * tj;
        T* q = P + r * w;
        for (int c = lane; c < wl; c += 32)
          if (c0 + c >= j) q[c] -= dsum * pr[c];
      }
    }
    __syncthreads();
  }
  // panel rows of W (this CTA's columns)
  for (int l = t; l < nbb * wl; l += bd) {
    const int r = l / wl, c = l - r * wl, gc = c0 + c;
    Wb[r * W.rs + gc * W.cs] = gc < r ? P[r * w + c] : (gc == r ? beta[r] : T(0));
  }
  __syncthreads();
  for (int l = t; l < nbb * wl; l += bd) {
    const int r = l / wl, c = l - r * wl;
    if (c0 + c < r) P[r * w + c] = T(0);
  }
  __syncthreads();
  // Gram matrix: partial sums here, summed over the cluster
  for (int pr_ = warp; pr_ < nbb * nbb; pr_ += nw) {
    const int i = pr_ / nbb, jj = pr_ - i * nbb;
    if (i >= jj) continue;
    T dsum = T(0);
    for (int c = lane; c < wl; c += 32) dsum += P[i * w + c] * P[jj * w + c];
    dsum = warp_sum(dsum);
    if (lane == 0) G[i][jj] = dsum;
  }
  cluster.sync();
  // (Gs sums the cluster's partials; G stays readable until the last barrier)
  __shared__ T Gs[kMaxPanel][kMaxPanel + 1];
  for (int l = t; l < nbb * nbb; l += bd) {
    const int i = l / nbb, jj = l - i * nbb;
    if (i < jj) {
      T g = T(0);
      for (int r = 0; r < CS; ++r) g += cluster.map_shared_rank(&G[0][0], r)[i * (kMaxPanel + 1) + jj];
      Gs[i][jj] = g;
    }
  }
  __syncthreads();
  if (warp == 0) {
    for (int jj = 0; jj < nbb; ++jj) {
      if (lane < jj) {
        T acc = T(0);
        for (int k = lane; k < jj; ++k) acc += Tm[lane][k] * Gs[k][jj];
        Tm[lane][jj] = -tau[jj] * acc;
      }
      if (lane == 0) Tm[jj][jj] = tau[jj];
      if (lane > jj && lane < nbb) Tm[lane][jj] = T(0);
      __syncwarp();
    }
  }
  __syncthreads();
  T* Vb = V + (int64_t)(blockIdx.x / CS) * vbs;
  T* TVb = TV + (int64_t)(blockIdx.x / CS) * vbs;
  for (int c = t; c < wl; c += bd) {
    for (int i = 0; i < nbb; ++i) {
      T acc = T(0);
      for (int k = i; k < nbb; ++k) acc = fma(Tm[i][k], P[k * w + c], acc);
      Vb[i * np + c0 + c] = P[i * w + c];
      TVb[i * np + c0 + c] = acc;
    }
  }
  cluster.sync();  // no CTA leaves while another may still read its shared memory
}

// ---------------------------------------------------------------------------
// Triangular solves.  op(L) X = B in place in B (M x K), L an M x M view that
// is lower triangular (`upper` == false) or upper triangular (a transposed
// lower view).  Few columns: k_trsv, one CTA per (column, batch entry),
// substitution with the right-hand side in shared memory.  Many columns:
// blocks of 32 rows, GEMM updates from the solved blocks and k_trsm_diag on
// the diagonal block (one thread per column).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_trsv(int M, MV<T> L, bool upper, MV<T> B, int64_t b0) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  T* x = s + M;
  const int t = threadIdx.x, bd = blockDim.x;
  const int64_t b = b0 + blockIdx.y;
  const T* Lb = L.p + b * L.bs;
  T* Bb = B.p + b * B.bs + blockIdx.x * B.cs;
  for (int i = t; i < M; i += bd) s[i] = Bb[i * B.rs];
  if (!upper) {
    for (int i = 0; i < M; ++i) {
      __syncthreads();
      const T xi = s[i] / Lb[i * L.rs + i * L.cs];
      for (int j = i + 1 + t; j < M; j += bd) s[j] -= Lb[j * L.rs + i * L.cs] * xi;
      if (t == 0) x[i] = xi;
    }
  } else {
    for (int i = M - 1; i >= 0; --i) {
      __syncthreads();
      const T xi = s[i] / Lb[i * L.rs + i * L.cs];
      for (int j = t; j < i; j += bd) s[j] -= Lb[j * L.rs + i * L.cs] * xi;
      if (t == 0) x[i] = xi;
    }
  }
  __syncthreads();
  for (int i = t; i < M; i += bd) Bb[i * B.rs] = x[i];
}

constexpr int kTrsmBlock = 32;

template <typename T>
__global__ void k_trsm_diag(int nbr, MV<T> L, bool upper, MV<T> B, int K, int64_t b0) {
  __shared__ T Ls[kTrsmBlock][kTrsmBlock + 1];
  const int t = threadIdx.x;
  const int64_t b = b0 + blockIdx.y;
  const T* Lb = L.p + b * L.bs;
  for (int l = t; l < nbr * nbr; l += blockDim.x) {
    const int i = l / nbr, j = l - i * nbr;
    Ls[i][j] = Lb[i * L.rs + j * L.cs];
  }
  __syncthreads();
  const int col = blockIdx.x * blockDim.x + t;
  if (col >= K) return;
  T* Bb = B.p + b * B.bs + col * B.cs;
  T x[kTrsmBlock];
#pragma unroll
  for (int i = 0; i < kTrsmBlock; ++i) x[i] = i < nbr ? Bb[i * B.rs] : T(0);
  if (!upper) {
#pragma unroll
    for (int i = 0; i < kTrsmBlock; ++i) {
      if (i < nbr) {
        T v = x[i];
#pragma unroll
        for (int j = 0; j < i; ++j) v -= Ls[i][j] * x[j];
        x[i] = v / Ls[i][i];
      }
    }
  } else {
#pragma unroll
    for (int i = kTrsmBlock - 1; i >= 0; --i) {
      if (i < nbr) {
        T v = x[i];
#pragma unroll
        for (int j = i + 1; j < kTrsmBlock; ++j)
          if (j < nbr) v -= Ls[i][j] * x[j];
        x[i] = v / Ls[i][i];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < kTrsmBlock; ++i)
    if (i < nbr) Bb[i * B.rs] = x[i];
}

// ---------------------------------------------------------------------------
// Elementwise: Y = alpha * X (+ beta * Y when beta != 0), a rows x cols block;
// fill a block with `v` off the diagonal and `dv` on it.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_axpby2d(int rows, int cols, T alpha, MV<T> X, T beta, MV<T> Y, int64_t b0) {
  const int64_t b = b0 + blockIdx.y;
  const int64_t n = (int64_t)rows * cols;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(l / cols), j = (int)(l - (int64_t)i * cols);
    T* y = Y.p + b * Y.bs + i * Y.rs + j * Y.cs;
    const T x = X.p[b * X.bs + i * X.rs + j * X.cs];
    *y = beta == T(0) ? alpha * x : fma(alpha, x, beta * *y);
  }
}

template <typename T>
__global__ void k_fill2d(int rows, int cols, T v, T dv, MV<T> Y, int64_t b0) {
  const int64_t b = b0 + blockIdx.y;
  const int64_t n = (int64_t)rows * cols;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(l / cols), j = (int)(l - (int64_t)i * cols);
    Y.p[b * Y.bs + i * Y.rs + j * Y.cs] = i == j ? dv : v;
  }
}

// Y = alpha F X + beta Y for a block-diagonal F (D x D, diagonal blocks of
// Q1 x Q1; the IWP transition I_d (x) A_1 in the state order of these
// kernels): each output sums the Q1 terms of its block, in the order a GEMM
// over the whole row would add them (the skipped products are exact zeros),
// so the result equals the dense product bit for bit.
template <typename T>
__global__ void k_blockdiag_mm(int D, int Q1, int K, MV<T> F, MV<T> X, T alpha, T beta, MV<T> Y, int64_t b0) {
  const int64_t b = b0 + blockIdx.y;
  const int64_t total = (int64_t)D * K;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < total; l += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(l / K), c = (int)(l - (int64_t)i * K);
    const int k0 = (i / Q1) * Q1;
    const T* Fr = F.p + b * F.bs + i * F.rs;
    const T* Xc = X.p + b * X.bs + c * X.cs;
    T acc = T(0);
    for (int k = k0; k < k0 + Q1; ++k) acc = fma(Fr[k * F.cs], Xc[k * X.rs], acc);
    T* y = Y.p + b * Y.bs + i * Y.rs + c * Y.cs;
    *y = beta == T(0) ? alpha * acc : fma(alpha, acc, beta * *y);
  }
}

// out[0] = number of non-zero entries of F (D x D) outside its diagonal
// Q1 x Q1 blocks (out[0] must be zero on entry).
template <typename T>
__global__ void k_offblock_count(int D, int Q1, const T* __restrict__ F, unsigned int* __restrict__ out) {
  unsigned int cnt = 0;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < (int64_t)D * D;
       l += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(l / D), j = (int)(l - (int64_t)i * D);
    if (i / Q1 != j / Q1 && F[l] != T(0)) ++cnt;
  }
  if (cnt) atomicAdd(out, cnt);
}

// Per-step filter terms from P11 (d x d lower), w = P11^{-1}(-r) and
// wq = P11^{-T} r: nll = |w|^2 / 2 + sum log|P11_ii| + d log(2 pi) / 2
// (pof/utils.py:22-30 negated), ssq = |wq|^2 (the whitened residual).
template <typename T>
__global__ void k_step_terms(int d, MV<T> P11, MV<T> w, MV<T> wq, double* __restrict__ nll,
                             double* __restrict__ ssq, int64_t stride, int64_t b0) {
  __shared__ double red[32];
  const int64_t b = b0 + blockIdx.x;
  double a = 0.0, q = 0.0, ld = 0.0;
  for (int i = threadIdx.x; i < d; i += blockDim.x) {
    const double wi = (double)w.p[b * w.bs + i * w.rs];
    const double qi = (double)wq.p[b * wq.bs + i * wq.rs];
    a += wi * wi;
    q += qi * qi;
    ld += log(fabs((double)P11.p[b * P11.bs + i * P11.rs + i * P11.cs]));
  }
  a = block_sum(a, red);
  q = block_sum(q, red);
  ld = block_sum(ld, red);
  if (threadIdx.x == 0) {
    nll[b * stride] = 0.5 * a + ld + 0.5 * d * 1.8378770664093453;  // log(2 pi)
    ssq[b * stride] = q;
  }
}

// out[b] = |x_b|^2 (x a vector of n entries per batch entry)
template <typename T>
__global__ void k_sqnorm(int n, MV<T> x, double* __restrict__ out, int64_t b0) {
  __shared__ double red[32];
  const int64_t b = b0 + blockIdx.x;
  double a = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = (double)x.p[b * x.bs + i * x.rs];
    a += v * v;
  }
  a = block_sum(a, red);
  if (threadIdx.x == 0) out[b] = a;
}

// Final scalars: sums of the per-step terms in chunk order (per chunk, then
// over chunks), written to out[POF_S_*]; ssq is divided by n * d.
__global__ void k_dense_scalars(const double* __restrict__ nll, const double* __restrict__ ssq,
                                const double* __restrict__ fobj, const double* __restrict__ sobj, int64_t n,
                                int64_t C0, int d, double* __restrict__ out, int which) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double sn = 0.0, ss = 0.0, sf = 0.0, so = 0.0;
  for (int64_t s = 0; s < n; s += C0) {
    const int64_t e = s + C0 < n ? s + C0 : n;
    double cn = 0.0, cs = 0.0, cf = 0.0, co = 0.0;
    for (int64_t k = s; k < e; ++k) {
      if (nll) cn += nll[k];
      if (ssq) cs += ssq[k];
      if (fobj) cf += fobj[k];
      if (sobj) co += sobj[k];
    }
    sn += cn;
    ss += cs;
    sf += cf;
    so += co;
  }
  if (which == 2) {  // smoothing alone
    out[1] = so;
    return;
  }
  out[0] = sn;
  out[2] = ss / (double)n / (double)d;
  out[3] = sf;
  out[1] = which == 0 ? sf : so;
  out[4] = 0.0;
}

}  // namespace dense
}  // namespace pof
