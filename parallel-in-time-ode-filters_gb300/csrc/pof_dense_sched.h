// The dense filter/smoother schedule (host code), written against a launch
// context X that provides the batched primitives on strided views:
//   gemm(batch, M, N, K, alpha, A, B, beta, C)     C = alpha A B + beta C
//   fmul(batch, K, F, X, alpha, beta, Y)           Y = alpha F X + beta Y with a
//                                                  transition matrix F (D x D): a
//                                                  GEMM, or the block-diagonal
//                                                  product when F has that form
//   axpby(batch, rows, cols, alpha, X, beta, Y)    Y = alpha X + beta Y
//   copy(batch, rows, cols, X, Y), fill(batch, rows, cols, v, diag_v, Y)
//   tria(batch, m, n, W)                           W (m x n, n >= m) -> L in
//                                                  its first m columns, zeros
//                                                  elsewhere (L L^T = W W^T)
//   trsm(batch, M, K, L, upper, B)                 op(L) X = B in place
//   step_terms(batch, d, P11, w, wq, nll, ssq, stride), sqnorm(batch, len, x, out),
//   scalars(nll, ssq, fobj, sobj, n, C0, d, out, which)
// pof_dense.cu runs it with CUDA kernels; tests/dense_sched_cpu.cpp runs the
// same code with host loops that check every access against the buffers.
#pragma once

#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "pof_dense_views.h"

namespace pof {
namespace dense {

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
constexpr size_t kSlabBytes = size_t(1) << 30;

// Bump allocation of the workspace; with base == nullptr it only sizes.
struct Arena {
  char* base;
  size_t off = 0;
  std::vector<std::pair<size_t, size_t>>* regions = nullptr;  // (offset, bytes) of every take, if wanted
  template <typename T>
  T* take(int64_t count) {
    off = (off + 255) & ~size_t(255);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    if (regions) regions->emplace_back(off, size_t(count) * sizeof(T));
    off += size_t(count) * sizeof(T);
    return p;
  }
};

// ---------------------------------------------------------------------------
// workspace layout (the same code sizes and carves it)
// ---------------------------------------------------------------------------
template <typename T>
struct Layout {
  int64_t n;
  int D, d, P, C0, last, S;
  int64_t maxbatch;
  // filter
  T *Ab[2], *Lc, *eta, *Z, *X1, *X2, *X3, *Gr;
  T *Sm, *SL, *Lk, *mk[2], *rb, *wb, *wq;
  // top levels (binary tree over the chunks): element and state slots of the
  // levels above the chunks (sum of the level sizes), and the scratch of one
  // batched operator application over at most G = ceil(P / 2) pairs
  T *TAb, *TU, *Teta, *TZ, *Sb, *SU;
  T *TgS, *TES, *TDS, *Em, *EL;
  T *OXi, *OM, *OT, *Om, *Oe, *OX5, *OX6, *Ov;
  int G;
  double *nll, *ssq, *fobj, *sobj;
  // smoother
  T *E, *Dm, *g, *Phi, *tE[2], *tD, *tg, *Xs, *em, *eL, *tm, *ftmp;
  // objectives
  T* R;
  // tria scratch
  T *V, *TV, *Y;
  int64_t vbs, ybs;
  unsigned int* flag;  // the block-structure check (zeroed by the caller)
  size_t total;

  // active chunks at step offset s of a chunk (only the last can be short)
  int active(int s) const { return s < last ? P : P - 1; }
};

// Default chunk count: the batch of every launch of the chunk loops.  float64
// is FP64-pipe bound from 64 chunks on at D = 640 (12.8 ms per step, 91 % of
// the FP64 rate); float32 is bound by the latency of each step's launch chain,
// so more chunks (fewer steps per chunk) keep paying up to ~256
// (reaction-diffusion, N = 4096: 5.5 s per pass at 64 chunks, 4.3 s at 256).
inline void plan_chunks(int64_t n, int chunks, int* P, int* C0, int* last, size_t es = 8) {
  int64_t p = chunks > 0 ? chunks : (es == 4 ? 256 : 64);
  const char* e = getenv("POF_DENSE_CHUNKS");
  if (chunks <= 0 && e && atoi(e) > 0) p = atoi(e);
  p = std::max<int64_t>(1, std::min<int64_t>(p, n));
  const int64_t c0 = cdiv(n, p);
  p = cdiv(n, c0);
  *P = (int)p;
  *C0 = (int)c0;
  *last = (int)(n - (p - 1) * c0);
}

template <typename T>
Layout<T> layout(char* base, int which, int64_t n, int D, int d, int chunks,
                 std::vector<std::pair<size_t, size_t>>* regions = nullptr) {
  Layout<T> L{};
  L.n = n;
  L.D = D;
  L.d = d;
  plan_chunks(n, chunks, &L.P, &L.C0, &L.last, sizeof(T));
  const int64_t P = L.P, DD = (int64_t)D * D;
  const int64_t es = sizeof(T);
  int64_t S = std::max<int64_t>(1, (int64_t)(kSlabBytes / (size_t(4 * DD) * es)));
  S = std::min<int64_t>(std::min<int64_t>(S, n), 4096);
  L.S = (int)S;
  Arena a{base};
  a.regions = regions;
  const bool filt = which != 2, smo = which != 0;
  // slots of the tree levels above the chunks: sum of n_{l+1} = ceil(n_l / 2)
  int64_t Tn = 0;
  for (int64_t m = P; m > 1; m = (m + 1) / 2) Tn += (m + 1) / 2;
  Tn = std::max<int64_t>(Tn, 1);
  if (filt) {
    L.Ab[0] = a.take<T>(P * D * (D + 1));
    L.Ab[1] = a.take<T>(P * D * (D + 1));
    L.Lc = a.take<T>(P * DD);
    L.eta = a.take<T>(P * D);
    L.Z = a.take<T>(P * DD);
    L.X1 = a.take<T>(P * D * 2 * D);
    L.X2 = a.take<T>(P * (int64_t)(D + d) * (D + d));
    L.X3 = a.take<T>(P * D * (int64_t)(D + d));
    L.Gr = a.take<T>(P * d * (int64_t)(D + 1));
    L.TAb = a.take<T>(Tn * D * (D + 1));
    L.TU = a.take<T>(Tn * DD);
    L.Teta = a.take<T>(Tn * D);
    L.TZ = a.take<T>(Tn * DD);
    L.Sb = a.take<T>(Tn * D);
    L.SU = a.take<T>(Tn * DD);
    L.Sm = a.take<T>(P * D);
    L.SL = a.take<T>(P * DD);
    L.Lk = a.take<T>(P * DD);
    L.mk[0] = a.take<T>(P * D);
    L.mk[1] = a.take<T>(P * D);
    L.rb = a.take<T>(P * d);
    L.wb = a.take<T>(P * d);
    L.wq = a.take<T>(P * d);
    L.nll = a.take<double>(n);
    L.ssq = a.take<double>(n);
    L.fobj = a.take<double>(n);
  }
  if (smo) {
    L.E = a.take<T>(n * DD);
    L.Dm = a.take<T>(n * DD);
    L.g = a.take<T>(n * D);
    L.Phi = a.take<T>(S * 4 * DD);
    L.tE[0] = a.take<T>(P * DD);
    L.tE[1] = a.take<T>(P * DD);
    L.tD = a.take<T>(P * DD);
    L.tg = a.take<T>(P * D);
    L.Xs = a.take<T>(P * 2 * DD);
    L.em = a.take<T>(P * D);
    L.eL = a.take<T>(P * DD);
    L.tm = a.take<T>(P * D);
    L.ftmp = a.take<T>(std::max<int64_t>(S, P) * D);
    L.sobj = a.take<double>(n);
    L.TgS = a.take<T>(Tn * D);
    L.TES = a.take<T>(Tn * DD);
    L.TDS = a.take<T>(Tn * DD);
    L.Em = a.take<T>(Tn * D);
    L.EL = a.take<T>(Tn * DD);
  }
  const int64_t G = std::max<int64_t>(1, (P + 1) / 2);
  L.G = (int)G;
  L.OXi = a.take<T>(G * 4 * DD);
  L.OM = a.take<T>(G * DD);
  L.OT = a.take<T>(G * DD);
  L.Om = a.take<T>(G * DD);
  L.Oe = a.take<T>(G * DD);
  L.OX5 = a.take<T>(G * 2 * DD);
  L.OX6 = a.take<T>(G * 2 * DD);
  L.Ov = a.take<T>(G * 8 * D);
  L.R = a.take<T>(n * D);
  const int nmax = std::max(2 * D, D + d), mmax = std::max(2 * D, D + d);
  L.maxbatch = std::max<int64_t>(P, S);
  L.vbs = (int64_t)kMaxPanel * nmax;
  L.ybs = (int64_t)mmax * kMaxPanel;
  L.V = a.take<T>(L.maxbatch * L.vbs);
  L.TV = a.take<T>(L.maxbatch * L.vbs);
  L.Y = a.take<T>(L.maxbatch * L.ybs);
  L.flag = reinterpret_cast<unsigned int*>(a.take<double>(1));
  L.total = a.off + 256;  // alignment slack of aligned_ws
  return L;
}

template <typename T>
struct Model {
  const T *F, *QL;
  int64_t fts;
  const T *H, *c, *R;
  int64_t rst;
};

template <typename T>
MV<T> cv(const T* p, int64_t rs, int64_t cs, int64_t bs) {
  return MV<T>{const_cast<T*>(p), rs, cs, bs};
}

// obj[k] = |QL_k^{-1} (M[k] - F_k M[k+1])|^2, k < n (pof/utils.py:97-101).
template <typename T, typename X>
void objective(X& cx, const Layout<T>& L, const T* F, const T* QL, int64_t fts, const T* M, double* obj) {
  const int D = L.D;
  const int64_t n = L.n;
  MV<T> Rv = rowmajor(L.R, D, 0);
  cx.copy(1, (int)n, D, cv(M, D, 1, 0), Rv);
  if (fts == 0) {
    cx.fmul(1, (int)n, cv(F, D, 1, 0), tr(cv(M + D, D, 1, 0)), T(-1), T(1), tr(Rv));
    cx.trsm(1, D, (int)n, cv(QL, D, 1, 0), false, tr(Rv));
  } else {
    MV<T> rv{L.R, 1, 1, D};
    cx.fmul(n, 1, cv(F, D, 1, fts), cv(M + D, 1, 1, D), T(-1), T(1), rv);
    cx.trsm(n, D, 1, cv(QL, D, 1, fts), false, rv);
  }
  cx.sqnorm(n, D, MV<T>{L.R, 1, 1, D}, obj);
}

// ---------------------------------------------------------------------------
// the top levels: a binary tree over the P chunk totals, the batched solve's
// segmented schedule with groups of two (restated by the oracle as
// blocked._filter_states_segmented / _smoother_states_segmented with Cg = 2).
// Level l has n_l elements (n_0 = P, n_{l+1} = ceil(n_l / 2)); the up-sweep
// combines the pairs (2g, 2g+1) of every level into the next, the down-sweep
// gives member 2g its parent's state and member 2g+1 that state carried
// through member 2g.  Every level is one batched application over its pairs.
// ---------------------------------------------------------------------------
template <typename T>
struct FElem {  // filter elements (A | b, U, eta, Z), one slot per element
  MV<T> Ab, U, eta, Z;
  FElem at(int64_t i) const {
    return FElem{MV<T>{Ab.p + i * Ab.bs, Ab.rs, Ab.cs, Ab.bs}, MV<T>{U.p + i * U.bs, U.rs, U.cs, U.bs},
                 MV<T>{eta.p + i * eta.bs, eta.rs, eta.cs, eta.bs}, MV<T>{Z.p + i * Z.bs, Z.rs, Z.cs, Z.bs}};
  }
  FElem pairs(int k) const {  // member k of every pair
    FElem e = at(k);
    e.Ab.bs *= 2, e.U.bs *= 2, e.eta.bs *= 2, e.Z.bs *= 2;
    return e;
  }
};

template <typename T>
struct State {  // (mean, chol) slots
  MV<T> m, L;
  State at(int64_t i) const {
    return State{MV<T>{m.p + i * m.bs, m.rs, m.cs, m.bs}, MV<T>{L.p + i * L.bs, L.rs, L.cs, L.bs}};
  }
  State pairs(int k) const {
    State s = at(k);
    s.m.bs *= 2, s.L.bs *= 2;
    return s;
  }
};

template <typename T>
struct SElem {  // smoother elements (g, E, D)
  MV<T> g, E, Dm;
  SElem at(int64_t i) const {
    return SElem{MV<T>{g.p + i * g.bs, g.rs, g.cs, g.bs}, MV<T>{E.p + i * E.bs, E.rs, E.cs, E.bs},
                 MV<T>{Dm.p + i * Dm.bs, Dm.rs, Dm.cs, Dm.bs}};
  }
  SElem pairs(int k) const {
    SElem e = at(k);
    e.g.bs *= 2, e.E.bs *= 2, e.Dm.bs *= 2;
    return e;
  }
};

template <typename T>
struct OpScratch {
  MV<T> Xi, M, Tm, m, e, X5, X6;
  MV<T> v[8];
  explicit OpScratch(const Layout<T>& L) {
    const int D = L.D;
    const int64_t DD = (int64_t)D * D;
    Xi = rowmajor(L.OXi, 2 * D, 4 * DD);
    M = rowmajor(L.OM, D, DD);
    Tm = rowmajor(L.OT, D, DD);
    m = rowmajor(L.Om, D, DD);
    e = rowmajor(L.Oe, D, DD);
    X5 = rowmajor(L.OX5, 2 * D, 2 * DD);
    X6 = rowmajor(L.OX6, 2 * D, 2 * DD);
    for (int i = 0; i < 8; ++i) v[i] = MV<T>{L.Ov + (int64_t)i * L.G * D, 1, 1, D};
  }
};

// Xi = tria([[U1^T Z2, I], [Z2, 0]]) and m = Xi11^{-1} U1^T (filter.py:117-142)
template <typename T, typename X>
void op_xi(X& cx, int D, int64_t G, MV<T> U1, MV<T> Z2, const OpScratch<T>& o) {
  const T one(1), zero(0);
  cx.gemm(G, D, D, D, one, tr(U1), Z2, zero, o.Xi);
  cx.fill(G, D, D, zero, one, sub(o.Xi, 0, D));
  cx.copy(G, D, D, Z2, sub(o.Xi, D, 0));
  cx.fill(G, D, D, zero, zero, sub(o.Xi, D, D));
  cx.tria(G, 2 * D, 2 * D, o.Xi);
  cx.copy(G, D, D, tr(U1), o.m);
  cx.trsm(G, D, D, o.Xi, false, o.m);
}

// b = A2 (I - m^T Xi21^T)(b1 + U1 U1^T eta2) + b2, written to out
template <typename T, typename X>
void op_b(X& cx, int D, int64_t G, MV<T> b1, MV<T> U1, MV<T> A2, MV<T> b2, MV<T> eta2, MV<T> out,
          const OpScratch<T>& o) {
  const T one(1), zero(0);
  const MV<T> Xi21 = sub(o.Xi, D, 0);
  cx.gemm(G, D, 1, D, one, tr(U1), eta2, zero, o.v[0]);
  cx.copy(G, D, 1, b1, o.v[1]);
  cx.gemm(G, D, 1, D, one, U1, o.v[0], one, o.v[1]);
  cx.gemm(G, D, 1, D, one, tr(Xi21), o.v[1], zero, o.v[2]);
  cx.copy(G, D, 1, o.v[1], o.v[3]);
  cx.gemm(G, D, 1, D, T(-1), tr(o.m), o.v[2], one, o.v[3]);
  cx.copy(G, D, 1, b2, out);
  cx.gemm(G, D, 1, D, one, A2, o.v[3], one, out);
}

// out = sqrt_filtering_operator(e1, e2) (filter.py:117-142), G pairs at once
template <typename T, typename X>
void op_filter(X& cx, int D, int64_t G, const FElem<T>& e1, const FElem<T>& e2, const FElem<T>& out,
               const OpScratch<T>& o) {
  const T one(1), zero(0);
  const MV<T> A1 = e1.Ab, b1 = sub(e1.Ab, 0, D), A2 = e2.Ab, b2 = sub(e2.Ab, 0, D);
  op_xi(cx, D, G, e1.U, e2.Z, o);
  const MV<T> Xi11 = o.Xi, Xi21 = sub(o.Xi, D, 0), Xi22 = sub(o.Xi, D, D);
  // M = Xi11^{-1} U1^T A2^T;  A = A2 A1 - M^T Xi21^T A1
  cx.gemm(G, D, D, D, one, tr(e1.U), tr(A2), zero, o.M);
  cx.trsm(G, D, D, Xi11, false, o.M);
  cx.gemm(G, D, D, D, one, tr(Xi21), A1, zero, o.Tm);
  cx.gemm(G, D, D, D, one, A2, A1, zero, out.Ab);
  cx.gemm(G, D, D, D, T(-1), tr(o.M), o.Tm, one, out.Ab);
  op_b(cx, D, G, b1, e1.U, A2, b2, e2.eta, sub(out.Ab, 0, D), o);
  // U = tria([M^T | U2])
  cx.copy(G, D, D, tr(o.M), o.X5);
  cx.copy(G, D, D, e2.U, sub(o.X5, 0, D));
  cx.tria(G, D, 2 * D, o.X5);
  cx.copy(G, D, D, o.X5, out.U);
  // eta = A1^T (I - e^T U1^T)(eta2 - Z2 Z2^T b1) + eta1,  e = Xi11^{-T} Xi21^T
  cx.copy(G, D, D, tr(Xi21), o.e);
  cx.trsm(G, D, D, tr(Xi11), true, o.e);
  cx.gemm(G, D, 1, D, one, tr(e2.Z), b1, zero, o.v[4]);
  cx.copy(G, D, 1, e2.eta, o.v[5]);
  cx.gemm(G, D, 1, D, T(-1), e2.Z, o.v[4], one, o.v[5]);
  cx.gemm(G, D, 1, D, one, tr(e1.U), o.v[5], zero, o.v[6]);
  cx.copy(G, D, 1, o.v[5], o.v[7]);
  cx.gemm(G, D, 1, D, T(-1), tr(o.e), o.v[6], one, o.v[7]);
  cx.copy(G, D, 1, e1.eta, out.eta);
  cx.gemm(G, D, 1, D, one, tr(A1), o.v[7], one, out.eta);
  // Z = tria([A1^T Xi22 | Z1])
  cx.gemm(G, D, D, D, one, tr(A1), Xi22, zero, o.X6);
  cx.copy(G, D, D, e1.Z, sub(o.X6, 0, D));
  cx.tria(G, D, 2 * D, o.X6);
  cx.copy(G, D, D, o.X6, out.Z);
}

// out = the (b, U) part of sqrt_filtering_operator((., b1, U1, ., .), e2):
// the filtering state after element e2 from the state (b1, U1) before it
template <typename T, typename X>
void op_propagate(X& cx, int D, int64_t G, const State<T>& s, const FElem<T>& e2, const State<T>& out,
                  const OpScratch<T>& o) {
  const T one(1), zero(0);
  const MV<T> A2 = e2.Ab, b2 = sub(e2.Ab, 0, D);
  op_xi(cx, D, G, s.L, e2.Z, o);
  op_b(cx, D, G, s.m, s.L, A2, b2, e2.eta, out.m, o);
  cx.gemm(G, D, D, D, one, A2, tr(o.m), zero, o.X5);
  cx.copy(G, D, D, e2.U, sub(o.X5, 0, D));
  cx.tria(G, D, 2 * D, o.X5);
  cx.copy(G, D, D, o.X5, out.L);
}

// state before every element of a level of n elements, the state before the
// first being given in st[top]; lev[l] / st[l] the levels' slots
template <typename T, typename X>
void filter_tree(X& cx, const Layout<T>& L, const FElem<T>& lev0, const State<T>& st0, const T* x0m, const T* x0L) {
  const int D = L.D;
  const int64_t DD = (int64_t)D * D;
  const OpScratch<T> o(L);
  std::vector<int64_t> n{L.P};
  while (n.back() > 1) n.push_back((n.back() + 1) / 2);
  const int top = (int)n.size() - 1;
  std::vector<FElem<T>> lev{lev0};
  std::vector<State<T>> st{st0};
  int64_t off = 0;
  for (int l = 1; l <= top; ++l) {
    lev.push_back(FElem<T>{rowmajor(L.TAb + off * D * (D + 1), D + 1, (int64_t)D * (D + 1)),
                           rowmajor(L.TU + off * DD, D, DD), MV<T>{L.Teta + off * D, 1, 1, D},
                           rowmajor(L.TZ + off * DD, D, DD)});
    st.push_back(State<T>{MV<T>{L.Sb + off * D, 1, 1, D}, rowmajor(L.SU + off * DD, D, DD)});
    off += n[l];
  }
  // up-sweep (the single top element is never needed)
  for (int l = 0; l + 1 < top; ++l) {
    const int64_t G2 = n[l] / 2;
    op_filter(cx, D, G2, lev[l].pairs(0), lev[l].pairs(1), lev[l + 1], o);
    if (n[l] % 2) {
      const FElem<T> a = lev[l].at(n[l] - 1), b = lev[l + 1].at(G2);
      cx.copy(1, D, D + 1, a.Ab, b.Ab);
      cx.copy(1, D, D, a.U, b.U);
      cx.copy(1, D, 1, a.eta, b.eta);
      cx.copy(1, D, D, a.Z, b.Z);
    }
  }
  cx.copy(1, D, 1, cv(x0m, 1, 1, 0), st[top].m);
  cx.copy(1, D, D, cv(x0L, D, 1, 0), st[top].L);
  // down-sweep
  for (int l = top - 1; l >= 0; --l) {
    const State<T> even = st[l].pairs(0);
    cx.copy(n[l + 1], D, 1, st[l + 1].m, even.m);
    cx.copy(n[l + 1], D, D, st[l + 1].L, even.L);
    op_propagate(cx, D, n[l] / 2, st[l + 1], lev[l].pairs(0), st[l].pairs(1), o);
  }
}

// smoothed state right after every chunk (the terminal state after the last)
template <typename T, typename X>
void smoother_tree(X& cx, const Layout<T>& L, const SElem<T>& lev0, const State<T>& ends0, const T* mT,
                   const T* LT) {
  const int D = L.D;
  const int64_t DD = (int64_t)D * D;
  const T one(1), zero(0);
  const OpScratch<T> o(L);
  std::vector<int64_t> n{L.P};
  while (n.back() > 1) n.push_back((n.back() + 1) / 2);
  const int top = (int)n.size() - 1;
  std::vector<SElem<T>> lev{lev0};
  std::vector<State<T>> en{ends0};
  int64_t off = 0;
  for (int l = 1; l <= top; ++l) {
    lev.push_back(SElem<T>{MV<T>{L.TgS + off * D, 1, 1, D}, rowmajor(L.TES + off * DD, D, DD),
                           rowmajor(L.TDS + off * DD, D, DD)});
    en.push_back(State<T>{MV<T>{L.Em + off * D, 1, 1, D}, rowmajor(L.EL + off * DD, D, DD)});
    off += n[l];
  }
  // up-sweep: the composite of every pair, sqrt_smoothing_operator(later, earlier)
  for (int l = 0; l + 1 < top; ++l) {
    const int64_t G2 = n[l] / 2;
    const SElem<T> early = lev[l].pairs(0), late = lev[l].pairs(1), out = lev[l + 1];
    cx.copy(G2, D, 1, early.g, out.g);
    cx.gemm(G2, D, 1, D, one, early.E, late.g, one, out.g);
    cx.gemm(G2, D, D, D, one, early.E, late.E, zero, out.E);
    cx.gemm(G2, D, D, D, one, early.E, late.Dm, zero, o.X5);
    cx.copy(G2, D, D, early.Dm, sub(o.X5, 0, D));
    cx.tria(G2, D, 2 * D, o.X5);
    cx.copy(G2, D, D, o.X5, out.Dm);
    if (n[l] % 2) {
      const SElem<T> a = lev[l].at(n[l] - 1), b = lev[l + 1].at(G2);
      cx.copy(1, D, 1, a.g, b.g);
      cx.copy(1, D, D, a.E, b.E);
      cx.copy(1, D, D, a.Dm, b.Dm);
    }
  }
  cx.copy(1, D, 1, cv(mT, 1, 1, 0), en[top].m);
  cx.copy(1, D, D, cv(LT, D, 1, 0), en[top].L);
  // down-sweep: member 2g+1 ends where its parent ends, member 2g where
  // member 2g+1 starts (the parent's end state carried through 2g+1)
  for (int l = top - 1; l >= 0; --l) {
    const int64_t G2 = n[l] / 2;
    const State<T> odd = en[l].pairs(1), even = en[l].pairs(0);
    const SElem<T> late = lev[l].pairs(1);
    cx.copy(G2, D, 1, en[l + 1].m, odd.m);
    cx.copy(G2, D, D, en[l + 1].L, odd.L);
    cx.copy(G2, D, 1, late.g, even.m);
    cx.gemm(G2, D, 1, D, one, late.E, en[l + 1].m, one, even.m);
    cx.gemm(G2, D, D, D, one, late.E, en[l + 1].L, zero, o.X5);
    cx.copy(G2, D, D, late.Dm, sub(o.X5, 0, D));
    cx.tria(G2, D, 2 * D, o.X5);
    cx.copy(G2, D, D, o.X5, even.L);
    if (n[l] % 2) {  // a last element alone in its pair ends where its parent ends
      const State<T> a = en[l + 1].at(G2), b = en[l].at(n[l] - 1);
      cx.copy(1, D, 1, a.m, b.m);
      cx.copy(1, D, D, a.L, b.L);
    }
  }
}

template <typename T, typename X>
void run_filter(X& cx, const Layout<T>& L, const Model<T>& md, const T* x0m, const T* x0L, T* om, T* oL) {
  const int D = L.D, d = L.d, P = L.P, C0 = L.C0;
  const int64_t DD = (int64_t)D * D;
  const T one(1), zero(0);
  auto Fv = [&](int s) { return cv(md.F + s * md.fts, D, 1, C0 * md.fts); };
  auto QLv = [&](int s) { return cv(md.QL + s * md.fts, D, 1, C0 * md.fts); };
  auto Hv = [&](int s) { return cv(md.H + (int64_t)s * d * D, D, 1, (int64_t)C0 * d * D); };
  auto cvec = [&](int s) { return cv(md.c + (int64_t)s * d, 1, 1, (int64_t)C0 * d); };
  auto Rv = [&](int s) { return cv(md.R + s * md.rst, d, 1, C0 * md.rst); };
  const MV<T> X1v = rowmajor(L.X1, 2 * D, 2 * DD);
  const MV<T> X2v = rowmajor(L.X2, D + d, (int64_t)(D + d) * (D + d));
  const MV<T> X3v = rowmajor(L.X3, D + d, (int64_t)D * (D + d));
  const MV<T> Grv = rowmajor(L.Gr, D + 1, (int64_t)d * (D + 1));
  const MV<T> Lcv = rowmajor(L.Lc, D, DD), Zv = rowmajor(L.Z, D, DD);
  const MV<T> etav{L.eta, 1, 1, D};
  MV<T> Abv[2] = {rowmajor(L.Ab[0], D + 1, (int64_t)D * (D + 1)), rowmajor(L.Ab[1], D + 1, (int64_t)D * (D + 1))};
  const MV<T> P11 = X2v, P21 = sub(X2v, d, 0), U = sub(X2v, d, d);

  // The X2 assembly [[H Lp, R], [Lp, 0]] from Lp = X1[:, :D] and its tria.
  auto observe = [&](int Pa, int s) {
    cx.gemm(Pa, d, D, D, one, Hv(s), X1v, zero, X2v);
    if (md.R)
      cx.copy(Pa, d, d, Rv(s), sub(X2v, 0, D));
    else
      cx.fill(Pa, d, d, zero, zero, sub(X2v, 0, D));
    cx.copy(Pa, D, D, X1v, sub(X2v, d, 0));
    cx.fill(Pa, D, d, zero, zero, sub(X2v, d, D));
    cx.tria(Pa, d + D, D + d, X2v);
  };
  auto predict = [&](int Pa, int s, MV<T> Lprev) {
    cx.fmul(Pa, D, Fv(s), Lprev, one, zero, X1v);
    cx.copy(Pa, D, D, QLv(s), sub(X1v, 0, D));
    cx.tria(Pa, D, 2 * D, X1v);
  };

  // phase 1: conditional fold of every chunk
  cx.fill(P, D, D + 1, zero, one, Abv[0]);
  cx.fill(P, D, D, zero, zero, Lcv);
  cx.fill(P, D, 1, zero, zero, etav);
  cx.fill(P, D, D, zero, zero, Zv);
  int cur = 0;
  for (int s = 0; s < C0; ++s) {
    const int Pa = L.active(s);
    predict(Pa, s, Lcv);
    observe(Pa, s);
    MV<T> FAb = Abv[1 - cur];
    cx.fmul(Pa, D + 1, Fv(s), Abv[cur], one, zero, FAb);
    cx.gemm(Pa, d, D + 1, D, one, Hv(s), FAb, zero, Grv);
    cx.axpby(Pa, d, 1, one, cvec(s), one, sub(Grv, 0, D));
    cx.trsm(Pa, d, D + 1, P11, false, Grv);
    cx.gemm(Pa, D, D + 1, d, T(-1), P21, Grv, one, FAb);
    // (a short last chunk's total may stay in the other buffer: phase 2
    // reads the totals of chunks 0..P-2 only, which are active every step)
    cur = 1 - cur;
    cx.gemm(Pa, D, 1, d, T(-1), tr(Grv), sub(Grv, 0, D), one, etav);
    cx.copy(Pa, D, D, Zv, X3v);
    cx.copy(Pa, D, d, tr(Grv), sub(X3v, 0, D));
    cx.tria(Pa, D, D + d, X3v);
    cx.copy(Pa, D, D, X3v, Zv);
    cx.copy(Pa, D, D, U, Lcv);
  }

  // phase 2: the state at every chunk start (the tree over the chunk totals)
  const MV<T> Smv{L.Sm, 1, 1, D}, SLv = rowmajor(L.SL, D, DD);
  filter_tree(cx, L, FElem<T>{Abv[cur], Lcv, etav, Zv}, State<T>{Smv, SLv}, x0m, x0L);

  // phase 3: the Kalman filter of every chunk from its start state
  const MV<T> Lkv = rowmajor(L.Lk, D, DD);
  MV<T> mkv[2] = {MV<T>{L.mk[0], 1, 1, D}, MV<T>{L.mk[1], 1, 1, D}};
  const MV<T> rbv{L.rb, 1, 1, d}, wbv{L.wb, 1, 1, d}, wqv{L.wq, 1, 1, d};
  cx.copy(P, D, D, SLv, Lkv);
  cx.copy(P, D, 1, Smv, mkv[0]);
  cx.copy(1, D, 1, cv(x0m, 1, 1, 0), MV<T>{om, 1, 1, 0});
  cx.copy(1, D, D, cv(x0L, D, 1, 0), rowmajor(oL, D, 0));
  cur = 0;
  for (int s = 0; s < C0; ++s) {
    const int Pa = L.active(s);
    predict(Pa, s, Lkv);
    MV<T> mp = mkv[1 - cur];
    cx.fmul(Pa, 1, Fv(s), mkv[cur], one, zero, mp);
    observe(Pa, s);
    cx.copy(Pa, d, 1, cvec(s), rbv);
    cx.gemm(Pa, d, 1, D, one, Hv(s), mp, one, rbv);
    cx.axpby(Pa, d, 1, T(-1), rbv, zero, wbv);
    cx.trsm(Pa, d, 1, P11, false, wbv);
    cx.copy(Pa, d, 1, rbv, wqv);
    cx.trsm(Pa, d, 1, tr(P11), true, wqv);
    cx.step_terms(Pa, d, P11, wbv, wqv, L.nll + s, L.ssq + s, C0);
    cx.gemm(Pa, D, 1, d, one, P21, wbv, one, mp);
    cx.copy(Pa, D, 1, mp, MV<T>{om + (int64_t)(s + 1) * D, 1, 1, (int64_t)C0 * D});
    cx.copy(Pa, D, D, U, rowmajor(oL + (s + 1) * DD, D, C0 * DD));
    cx.copy(Pa, D, D, U, Lkv);
    cur = 1 - cur;
  }
  objective(cx, L, md.F, md.QL, md.fts, om, L.fobj);
}

template <typename T, typename X>
void run_smoother(X& cx, const Layout<T>& L, const T* F, const T* QL, int64_t fts, T* om, T* oL) {
  const int D = L.D, P = L.P, C0 = L.C0;
  const int64_t n = L.n, DD = (int64_t)D * D;
  const T one(1), zero(0);
  // elements (g, E, D) of every step, in slabs of S steps
  const MV<T> Phiv = rowmajor(L.Phi, 2 * D, 4 * DD);
  for (int64_t k0 = 0; k0 < n; k0 += L.S) {
    const int64_t Sb = std::min<int64_t>(L.S, n - k0);
    const MV<T> Fk = cv(F + k0 * fts, D, 1, fts), QLk = cv(QL + k0 * fts, D, 1, fts);
    const MV<T> Lk = rowmajor(oL + k0 * DD, D, DD);
    const MV<T> mk{om + k0 * D, 1, 1, D};
    const MV<T> Ek = rowmajor(L.E + k0 * DD, D, DD), Dk = rowmajor(L.Dm + k0 * DD, D, DD);
    const MV<T> gk{L.g + k0 * D, 1, 1, D}, ft{L.ftmp, 1, 1, D};
    cx.fmul(Sb, D, Fk, Lk, one, zero, Phiv);
    cx.copy(Sb, D, D, QLk, sub(Phiv, 0, D));
    cx.copy(Sb, D, D, Lk, sub(Phiv, D, 0));
    cx.fill(Sb, D, D, zero, zero, sub(Phiv, D, D));
    cx.tria(Sb, 2 * D, 2 * D, Phiv);
    cx.trsm(Sb, D, D, tr(Phiv), true, tr(sub(Phiv, D, 0)));  // P21 block := E = P21 P11^{-1}
    cx.copy(Sb, D, D, sub(Phiv, D, 0), Ek);
    cx.copy(Sb, D, D, sub(Phiv, D, D), Dk);
    cx.fmul(Sb, 1, Fk, mk, one, zero, ft);
    cx.copy(Sb, D, 1, mk, gk);
    cx.gemm(Sb, D, 1, D, T(-1), Ek, ft, one, gk);
  }
  auto Ev = [&](int off) { return rowmajor(L.E + off * DD, D, C0 * DD); };
  auto Dv = [&](int off) { return rowmajor(L.Dm + off * DD, D, C0 * DD); };
  auto gv = [&](int off) { return MV<T>{L.g + (int64_t)off * D, 1, 1, (int64_t)C0 * D}; };
  MV<T> tEv[2] = {rowmajor(L.tE[0], D, DD), rowmajor(L.tE[1], D, DD)};
  const MV<T> tDv = rowmajor(L.tD, D, DD), tgv{L.tg, 1, 1, D};
  const MV<T> Xsv = rowmajor(L.Xs, 2 * D, 2 * DD);
  // composite of every chunk's elements (sqrt_smoothing_operator, later
  // element first).  The product E_tot E_i goes to scratch and is copied
  // back, so a short last chunk keeps its total in place while the others
  // go on.
  cx.copy(P, D, D, Ev(0), tEv[0]);
  cx.copy(P, D, D, Dv(0), tDv);
  cx.copy(P, D, 1, gv(0), tgv);
  for (int off = 1; off < C0; ++off) {
    const int Pa = L.active(off);
    cx.gemm(Pa, D, D, D, one, tEv[0], Ev(off), zero, tEv[1]);
    cx.gemm(Pa, D, 1, D, one, tEv[0], gv(off), one, tgv);
    cx.gemm(Pa, D, D, D, one, tEv[0], Dv(off), zero, Xsv);
    cx.copy(Pa, D, D, tDv, sub(Xsv, 0, D));
    cx.tria(Pa, D, 2 * D, Xsv);
    cx.copy(Pa, D, D, Xsv, tDv);
    cx.copy(Pa, D, D, tEv[1], tEv[0]);
  }
  // smoothed state at every chunk end, from the terminal (filtered) state
  const MV<T> emv{L.em, 1, 1, D}, eLv = rowmajor(L.eL, D, DD);
  smoother_tree(cx, L, SElem<T>{tgv, tEv[0], tDv}, State<T>{emv, eLv}, om + n * D, oL + n * DD);
  // backward recursion inside every chunk
  const MV<T> tmv{L.tm, 1, 1, D};
  for (int off = C0 - 1; off >= 0; --off) {
    const int Pa = L.active(off);
    cx.copy(Pa, D, 1, gv(off), tmv);
    cx.gemm(Pa, D, 1, D, one, Ev(off), emv, one, tmv);
    cx.gemm(Pa, D, D, D, one, Ev(off), eLv, zero, Xsv);
    cx.copy(Pa, D, D, Dv(off), sub(Xsv, 0, D));
    cx.tria(Pa, D, 2 * D, Xsv);
    cx.copy(Pa, D, 1, tmv, MV<T>{om + (int64_t)off * D, 1, 1, (int64_t)C0 * D});
    cx.copy(Pa, D, D, Xsv, rowmajor(oL + off * DD, D, C0 * DD));
    cx.copy(Pa, D, 1, tmv, emv);
    cx.copy(Pa, D, D, Xsv, eLv);
  }
  objective(cx, L, F, QL, fts, om, L.sobj);
}


// The whole pass: which = 0 filter, 1 filter + smoother, 2 smoother (x0m /
// x0L are the filtered means / chols, copied to om / oL first).
template <typename T, typename X>
void run_schedule(X& cx, const Layout<T>& L, int which, const T* x0m, const T* x0L, const T* F, const T* QL,
                  int64_t fts, const T* H, const T* c, const T* R, int64_t rst, T* om, T* oL, double* osc) {
  const int D = L.D;
  const int64_t n = L.n;
  if (which != 2) {
    Model<T> md{F, QL, fts, H, c, R, R ? rst : 0};
    run_filter(cx, L, md, x0m, x0L, om, oL);
  } else {
    if (om != x0m) cx.copy(1, (int)(n + 1), D, cv(x0m, D, 1, 0), rowmajor(om, D, 0));
    if (oL != x0L) cx.copy(1, (int)((n + 1) * D), D, cv(x0L, D, 1, 0), rowmajor(oL, D, 0));
  }
  if (which != 0) run_smoother(cx, L, F, QL, fts, om, oL);
  if (osc) cx.scalars(L.nll, L.ssq, L.fobj, L.sobj, n, L.C0, L.d, osc, which);
}

}  // namespace dense
}  // namespace pof
