// The dense filter/smoother schedule (csrc/pof_dense_sched.h) run on the
// host, with every primitive written as plain loops and every element access
// checked against the buffers it may touch: the workspace (filled with NaN
// first, so reading scratch that was never written shows up as NaN in the
// results), the inputs (read only) and the outputs.  Built as a shared
// library by tests/test_dense_cpu.py and compared there with the NumPy
// oracle's segmented schedule; the CUDA kernels replace these loops on the
// GPU, under the same views and sizes.
//
//   int dense_cpu_filtsmooth(which, n, D, d, x0m, x0L, F, QL, fts, H, c, R,
//                            rst, om, oL, osc, chunks, msg, msg_len)
// returns 0, or -1 with the first out-of-bounds access described in msg.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <limits>
#include <string>
#include <vector>

#include "pof_dense_sched.h"

using namespace pof::dense;

namespace {

struct Range {
  const char* name;
  const double* lo;
  int64_t count;
  bool writable;
};

struct CpuCtx {
  std::vector<Range> ranges;
  std::string err;
  const char* op = "";

  // p must lie in the buffer (a workspace region of the layout, an input or
  // an output) that holds `base`, the first element of the view it is read
  // through: an index running past its own buffer into a neighbour is caught
  bool ok(const double* p, bool write, const double* base = nullptr) {
    if (!base) base = p;
    for (const Range& r : ranges)
      if (base >= r.lo && base < r.lo + r.count) {
        if (p >= r.lo && p < r.lo + r.count && !(write && !r.writable)) return true;
        break;
      }
    if (err.empty()) {
      char buf[256];
      snprintf(buf, sizeof buf, "%s: %s access at %p outside the buffer of its view (base %p)", op,
               write ? "write" : "read", (const void*)p, (const void*)base);
      err = buf;
    }
    return false;
  }
  double get(const MV<double>& a, int64_t b, int64_t i, int64_t j) {
    const double* p = a.p + b * a.bs + i * a.rs + j * a.cs;
    return ok(p, false, a.p) ? *p : std::numeric_limits<double>::quiet_NaN();
  }
  void put(const MV<double>& a, int64_t b, int64_t i, int64_t j, double v) {
    double* p = a.p + b * a.bs + i * a.rs + j * a.cs;
    if (ok(p, true, a.p)) *p = v;
  }

  void gemm(int64_t batch, int M, int N, int K, double alpha, MV<double> A, MV<double> B, double beta,
            MV<double> C) {
    op = "gemm";
    std::vector<double> acc((size_t)M * N);
    for (int64_t b = 0; b < batch; ++b) {
      for (int i = 0; i < M; ++i)
        for (int j = 0; j < N; ++j) {
          double s = 0.0;
          for (int k = 0; k < K; ++k) s += get(A, b, i, k) * get(B, b, k, j);
          acc[(size_t)i * N + j] = s;
        }
      for (int i = 0; i < M; ++i)
        for (int j = 0; j < N; ++j) {
          const double v = alpha * acc[(size_t)i * N + j];
          put(C, b, i, j, beta == 0.0 ? v : v + beta * get(C, b, i, j));
        }
    }
  }
  int D = 0;
  void fmul(int64_t batch, int K, MV<double> F, MV<double> X, double alpha, double beta, MV<double> Y) {
    gemm(batch, D, K, D, alpha, F, X, beta, Y);
  }
  void axpby(int64_t batch, int rows, int cols, double alpha, MV<double> X, double beta, MV<double> Y) {
    op = "axpby";
    for (int64_t b = 0; b < batch; ++b)
      for (int i = 0; i < rows; ++i)
        for (int j = 0; j < cols; ++j) {
          const double v = alpha * get(X, b, i, j);
          put(Y, b, i, j, beta == 0.0 ? v : v + beta * get(Y, b, i, j));
        }
  }
  void copy(int64_t batch, int rows, int cols, MV<double> X, MV<double> Y) { axpby(batch, rows, cols, 1.0, X, 0.0, Y); }
  void fill(int64_t batch, int rows, int cols, double v, double dv, MV<double> Y) {
    op = "fill";
    for (int64_t b = 0; b < batch; ++b)
      for (int i = 0; i < rows; ++i)
        for (int j = 0; j < cols; ++j) put(Y, b, i, j, i == j ? dv : v);
  }
  // unblocked Householder LQ, dlarfg convention; row i ends as
  // [L entries, beta, 0 ... 0]
  void tria(int64_t batch, int m, int n, MV<double> W) {
    op = "tria";
    if (n < m && err.empty()) err = "tria: n < m";
    std::vector<double> v(n);
    for (int64_t b = 0; b < batch; ++b)
      for (int i = 0; i < m; ++i) {
        double s = 0.0;
        for (int c = i + 1; c < n; ++c) {
          const double x = get(W, b, i, c);
          s += x * x;
        }
        const double alpha = get(W, b, i, i);
        double beta, tau, scale;
        if (s == 0.0) {
          tau = 0.0;
          beta = alpha;
          scale = 0.0;
        } else {
          const double h = hypot(alpha, sqrt(s));
          beta = alpha >= 0.0 ? -h : h;
          tau = (beta - alpha) / beta;
          scale = 1.0 / (alpha - beta);
        }
        v[i] = 1.0;
        for (int c = i + 1; c < n; ++c) v[c] = get(W, b, i, c) * scale;
        if (tau != 0.0)
          for (int r = i + 1; r < m; ++r) {
            double dsum = 0.0;
            for (int c = i; c < n; ++c) dsum += get(W, b, r, c) * v[c];
            dsum *= tau;
            for (int c = i; c < n; ++c) put(W, b, r, c, get(W, b, r, c) - dsum * v[c]);
          }
        put(W, b, i, i, beta);
        for (int c = i + 1; c < n; ++c) put(W, b, i, c, 0.0);
      }
  }
  void trsm(int64_t batch, int M, int K, MV<double> L, bool upper, MV<double> B) {
    op = "trsm";
    for (int64_t b = 0; b < batch; ++b)
      for (int k = 0; k < K; ++k) {
        if (!upper) {
          for (int i = 0; i < M; ++i) {
            double s = get(B, b, i, k);
            for (int j = 0; j < i; ++j) s -= get(L, b, i, j) * get(B, b, j, k);
            put(B, b, i, k, s / get(L, b, i, i));
          }
        } else {
          for (int i = M - 1; i >= 0; --i) {
            double s = get(B, b, i, k);
            for (int j = i + 1; j < M; ++j) s -= get(L, b, i, j) * get(B, b, j, k);
            put(B, b, i, k, s / get(L, b, i, i));
          }
        }
      }
  }
  void step_terms(int64_t batch, int d, MV<double> P11, MV<double> w, MV<double> wq, double* nll, double* ssq,
                  int64_t stride) {
    op = "step_terms";
    for (int64_t b = 0; b < batch; ++b) {
      double a = 0.0, q = 0.0, ld = 0.0;
      for (int i = 0; i < d; ++i) {
        const double wi = get(w, b, i, 0), qi = get(wq, b, i, 0);
        a += wi * wi;
        q += qi * qi;
        ld += log(fabs(get(P11, b, i, i)));
      }
      if (ok(nll + b * stride, true)) nll[b * stride] = 0.5 * a + ld + 0.5 * d * 1.8378770664093453;
      if (ok(ssq + b * stride, true)) ssq[b * stride] = q;
    }
  }
  void sqnorm(int64_t batch, int len, MV<double> x, double* out) {
    op = "sqnorm";
    for (int64_t b = 0; b < batch; ++b) {
      double a = 0.0;
      for (int i = 0; i < len; ++i) {
        const double v = get(x, b, i, 0);
        a += v * v;
      }
      if (ok(out + b, true)) out[b] = a;
    }
  }
  void scalars(const double* nll, const double* ssq, const double* fobj, const double* sobj, int64_t n, int64_t C0,
               int d, double* out, int which) {
    op = "scalars";
    double sn = 0.0, ss = 0.0, sf = 0.0, so = 0.0;
    for (int64_t k = 0; k < n; ++k) {
      if (nll && ok(nll + k, false)) sn += nll[k];
      if (ssq && ok(ssq + k, false)) ss += ssq[k];
      if (fobj && ok(fobj + k, false)) sf += fobj[k];
      if (sobj && ok(sobj + k, false)) so += sobj[k];
    }
    (void)C0;
    if (which == 2) {
      out[1] = so;
      return;
    }
    out[0] = sn;
    out[2] = ss / (double)n / (double)d;
    out[3] = sf;
    out[1] = which == 0 ? sf : so;
    out[4] = 0.0;
  }
};

}  // namespace

extern "C" int dense_cpu_workspace_check(int which, int64_t n, int D, int d, int chunks, int64_t* out) {
  Layout<double> L = layout<double>(nullptr, which, n, D, d, chunks);
  out[0] = (int64_t)L.total;
  out[1] = L.P;
  out[2] = L.C0;
  out[3] = L.last;
  out[4] = L.S;
  return 0;
}

extern "C" int dense_cpu_filtsmooth(int which, int64_t n, int D, int d, const double* x0m, const double* x0L,
                                    const double* F, const double* QL, int64_t fts, const double* H,
                                    const double* c, const double* R, int64_t rst, double* om, double* oL,
                                    double* osc, int chunks, char* msg, int msg_len) {
  Layout<double> sz = layout<double>(nullptr, which, n, D, d, chunks);
  std::vector<double> ws(sz.total / sizeof(double) + 64, std::numeric_limits<double>::quiet_NaN());
  char* base = reinterpret_cast<char*>(ws.data());
  char* al = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(base) + 255) & ~uintptr_t(255));
  std::vector<std::pair<size_t, size_t>> regions;
  Layout<double> L = layout<double>(al, which, n, D, d, chunks, &regions);
  CpuCtx cx;
  cx.D = D;
  const int64_t DD = (int64_t)D * D;
  const int64_t ft_count = fts ? n * DD : DD;
  for (const auto& r : regions)
    cx.ranges.push_back({"workspace", reinterpret_cast<const double*>(al + r.first),
                         (int64_t)(r.second / sizeof(double)), true});
  if (which != 2) {
    cx.ranges.push_back({"x0m", x0m, D, false});
    cx.ranges.push_back({"x0L", x0L, DD, false});
    cx.ranges.push_back({"H", H, n * d * D, false});
    cx.ranges.push_back({"c", c, n * d, false});
    if (R) cx.ranges.push_back({"R", R, rst ? n * d * d : (int64_t)d * d, false});
  } else {
    cx.ranges.push_back({"filt_mean", x0m, (n + 1) * D, false});
    cx.ranges.push_back({"filt_chol", x0L, (n + 1) * DD, false});
  }
  cx.ranges.push_back({"F", F, ft_count, false});
  cx.ranges.push_back({"QL", QL, ft_count, false});
  cx.ranges.push_back({"om", om, (n + 1) * D, true});
  cx.ranges.push_back({"oL", oL, (n + 1) * DD, true});
  cx.ranges.push_back({"osc", osc, 8, true});
  run_schedule<double>(cx, L, which, x0m, x0L, F, QL, fts, H, c, R, rst, om, oL, osc);
  if (!cx.err.empty()) {
    snprintf(msg, msg_len, "%s", cx.err.c_str());
    return -1;
  }
  return 0;
}
