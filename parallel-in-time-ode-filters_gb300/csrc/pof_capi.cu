// C ABI of libpof.so (declared in include/pof.h).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/pof.h"
#include "pof_table.cuh"

using namespace pof;

namespace {

thread_local std::string g_cuda_error;

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return POF_OK;
  g_cuda_error = cudaGetErrorString(e);
  return POF_ERR_CUDA;
}

int launch_status() { return cuda_status(cudaGetLastError()); }

const Ops* find_ops(int dtype, int D, int DY) {
  if (dtype != POF_F64 && dtype != POF_F32) return nullptr;
  if (DY < 1 || D % DY != 0) return nullptr;
  return find_shape(dtype, D, DY);
}

int esz(int dtype) { return dtype == POF_F32 ? 4 : 8; }

// Optional overrides of the chunk sizes (tuning): POF_C0, POF_CG.
int env_int(const char* name) {
  const char* v = getenv(name);
  return v ? atoi(v) : 0;
}

Plan plan_for(int dtype, int64_t n, int D, int DY, bool solver) {
  return make_plan(n, D, DY, esz(dtype), solver, env_int("POF_C0"), env_int("POF_CG"));
}

int check_common(int dtype, int64_t n, int D, int DY, const Ops** ops) {
  if (dtype != POF_F64 && dtype != POF_F32) return POF_ERR_DTYPE;
  if (n < 1 || D < 1 || DY < 1 || DY > D) return POF_ERR_ARG;
  *ops = find_ops(dtype, D, DY);
  if (!*ops) return POF_ERR_SHAPE;
  return POF_OK;
}

// The filter's scalars are reported through the same block layout.
void report_scalars(const Plan& p, char* ws, double* out, cudaStream_t st) {
  if (out) k_copy_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(ws + p.scalars), out, 0);
}

char* aligned_ws(void* ws) {
  uintptr_t a = reinterpret_cast<uintptr_t>(ws);
  a = (a + 255) & ~uintptr_t(255);
  return reinterpret_cast<char*>(a);
}

// ---------------------------------------------------------------------------
// Per-kernel timing (pof_profile_*): event pairs from a pool, recorded on
// the launching stream, summed per kind when collected.  Single host thread.
// ---------------------------------------------------------------------------
struct ProfPair {
  int kind;
  cudaEvent_t b, e;
};
struct ProfState {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  std::vector<ProfPair> open, done;
  double ms[PK_COUNT] = {0};
  int64_t count[PK_COUNT] = {0};
};
ProfState g_prof;

cudaEvent_t prof_event() {
  if (!g_prof.pool.empty()) {
    cudaEvent_t e = g_prof.pool.back();
    g_prof.pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

void prof_collect() {
  for (const ProfPair& pp : g_prof.done) {
    float ms = 0.f;
    if (cudaEventSynchronize(pp.e) == cudaSuccess && cudaEventElapsedTime(&ms, pp.b, pp.e) == cudaSuccess) {
      g_prof.ms[pp.kind] += ms;
      g_prof.count[pp.kind] += 1;
    }
    g_prof.pool.push_back(pp.b);
    g_prof.pool.push_back(pp.e);
  }
  g_prof.done.clear();
}

}  // namespace

namespace pof {
bool prof_on() { return g_prof.on; }
void prof_begin(int kind, cudaStream_t st) {
  ProfPair pp{kind, prof_event(), prof_event()};
  cudaEventRecord(pp.b, st);
  g_prof.open.push_back(pp);
}
void prof_end(int kind, cudaStream_t st) {
  for (size_t i = g_prof.open.size(); i-- > 0;) {
    if (g_prof.open[i].kind == kind) {
      cudaEventRecord(g_prof.open[i].e, st);
      g_prof.done.push_back(g_prof.open[i]);
      g_prof.open.erase(g_prof.open.begin() + i);
      return;
    }
  }
}
}  // namespace pof

extern "C" {

// FP64 FMA throughput probe: 8 independent dependency chains per thread.
__global__ void k_fp64_probe(int64_t iters, double* sink) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double b = 0.999999999, c = 1e-12;
  for (int64_t i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  const double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) sink[blockIdx.x] = s;  // keeps the chains alive
}

int pof_fp64_probe(int64_t iters, int32_t blocks, int32_t threads, double* sink, void* stream) {
  if (iters < 1 || blocks < 1 || threads < 1 || threads > 1024 || !sink) return POF_ERR_ARG;
  k_fp64_probe<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(iters, sink);
  return launch_status();
}

void pof_profile_enable(int32_t on) {
  prof_collect();
  g_prof.on = on != 0;
}

int pof_profile_read(double* ms_out, int64_t* count_out, int32_t nkinds, int32_t reset) {
  prof_collect();
  const int k = nkinds < PK_COUNT ? nkinds : PK_COUNT;
  for (int i = 0; i < k; ++i) {
    if (ms_out) ms_out[i] = g_prof.ms[i];
    if (count_out) count_out[i] = g_prof.count[i];
  }
  if (reset) {
    for (int i = 0; i < PK_COUNT; ++i) {
      g_prof.ms[i] = 0.0;
      g_prof.count[i] = 0;
    }
  }
  return PK_COUNT;
}

const char* pof_status_string(int status) {
  switch (status) {
    case POF_OK: return "ok";
    case POF_ERR_ARG: return "invalid argument";
    case POF_ERR_SHAPE: return "(D, d) combination not compiled into libpof";
    case POF_ERR_WORKSPACE: return "workspace too small";
    case POF_ERR_CUDA: return "CUDA runtime error";
    case POF_ERR_FIELD: return "unknown built-in field or dimension mismatch";
    case POF_ERR_DTYPE: return "unsupported dtype";
    default: return "unknown status";
  }
}

const char* pof_last_cuda_error(void) { return g_cuda_error.c_str(); }

int pof_version(void) { return 1; }

int pof_shape_supported(int32_t D, int32_t d) { return find_ops(POF_F64, D, d) != nullptr ? 1 : 0; }

size_t pof_filtsmooth_workspace_bytes(int32_t dtype, int64_t n_steps, int32_t D, int32_t d) {
  if (n_steps < 1 || D < 1) return 0;
  return plan_for(dtype, n_steps, D, d, false).total;
}

size_t pof_ieks_workspace_bytes(int32_t dtype, int64_t n_steps, int32_t D, int32_t d) {
  if (n_steps < 1 || D < 1) return 0;
  return plan_for(dtype, n_steps, D, d, true).total;
}

static int filtsmooth_impl(int which, int32_t dtype, int64_t n, int32_t D, int32_t d, const void* x0m,
                           const void* x0L, const void* F, const void* QL, int64_t fts, const void* H,
                           const void* c, const void* R, int64_t rs, void* om, void* oL, double* osc, void* ws,
                           size_t wsb, void* stream) {
  const Ops* ops = nullptr;
  int rc = check_common(dtype, n, D, d, &ops);
  if (rc) return rc;
  if (!x0m || !x0L || !F || !QL || !H || !c || !om || !oL || !ws) return POF_ERR_ARG;
  if (fts != 0 && fts != (int64_t)D * D) return POF_ERR_ARG;
  if (R && rs != 0 && rs != (int64_t)d * d) return POF_ERR_ARG;
  Plan p = plan_for(dtype, n, D, d, false);
  if (wsb < p.total) return POF_ERR_WORKSPACE;
  char* w = aligned_ws(ws);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  StepModel sm{F, QL, fts, H, c, R, rs};
  k_init_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(w + p.scalars));
  ops->filter(p, w, sm, x0m, x0L, om, oL, st);
  if (which == 1) ops->smoother(p, w, F, QL, fts, om, oL, false, nullptr, st);
  report_scalars(p, w, osc, st);
  if (which == 0 && osc) {
    // linear_noiseless_filtering returns the filter objective as `obj`
    cudaError_t e = cudaMemcpyAsync(osc + POF_S_OBJ, osc + POF_S_FOBJ, sizeof(double), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return launch_status();
}

int pof_linear_filtsmooth(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, const void* x0_mean,
                          const void* x0_chol, const void* F, const void* QL, int64_t ft_stride, const void* H,
                          const void* c, const void* R, int64_t r_stride, void* out_mean, void* out_chol,
                          double* out_scalars, void* workspace, size_t workspace_bytes, void* stream) {
  return filtsmooth_impl(1, dtype, n_steps, D, d, x0_mean, x0_chol, F, QL, ft_stride, H, c, R, r_stride, out_mean,
                         out_chol, out_scalars, workspace, workspace_bytes, stream);
}

int pof_linear_noiseless_filtering(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, const void* x0_mean,
                                   const void* x0_chol, const void* F, const void* QL, int64_t ft_stride,
                                   const void* H, const void* c, const void* R, int64_t r_stride, void* out_mean,
                                   void* out_chol, double* out_scalars, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  return filtsmooth_impl(0, dtype, n_steps, D, d, x0_mean, x0_chol, F, QL, ft_stride, H, c, R, r_stride, out_mean,
                         out_chol, out_scalars, workspace, workspace_bytes, stream);
}

int pof_smoothing(int32_t dtype, int64_t n_steps, int32_t D, const void* F, const void* QL, int64_t ft_stride,
                  const void* filt_mean, const void* filt_chol, void* out_mean, void* out_chol, double* out_scalars,
                  void* workspace, size_t workspace_bytes, void* stream) {
  // The smoother does not depend on d; use the d = 1 instantiation when D
  // allows, else any compiled d dividing D.
  const Ops* ops = nullptr;
  int dy_used = 0;
  for (int dy = 1; dy <= 4 && !ops; ++dy) {
    if (D % dy == 0) {
      ops = find_ops(dtype, D, dy);
      dy_used = dy;
    }
  }
  if (dtype != POF_F64 && dtype != POF_F32) return POF_ERR_DTYPE;
  if (!ops) return POF_ERR_SHAPE;
  if (n_steps < 1 || !F || !QL || !filt_mean || !filt_chol || !out_mean || !out_chol || !workspace)
    return POF_ERR_ARG;
  if (ft_stride != 0 && ft_stride != (int64_t)D * D) return POF_ERR_ARG;
  Plan p = plan_for(dtype, n_steps, D, dy_used, false);
  if (workspace_bytes < p.total) return POF_ERR_WORKSPACE;
  char* w = aligned_ws(workspace);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t es = esz(dtype);
  k_init_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(w + p.scalars));
  if (out_mean != filt_mean) {
    cudaError_t e = cudaMemcpyAsync(out_mean, filt_mean, es * D * (n_steps + 1), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  if (out_chol != filt_chol) {
    cudaError_t e =
        cudaMemcpyAsync(out_chol, filt_chol, es * D * D * (n_steps + 1), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  ops->smo_elements(n_steps, F, QL, ft_stride, out_mean, out_chol, w + p.selem, st);
  ops->smoother(p, w, F, QL, ft_stride, out_mean, out_chol, false, nullptr, st);
  report_scalars(p, w, out_scalars, st);
  return launch_status();
}

static int nordsieck_p01(int D, int d, double h, double* p0, double* p1) {
  const int q = D / d - 1;
  if (q < 1 || D % d) return POF_ERR_ARG;
  // P = diag(|h|^(q-i+1/2) / (q-i)!), i = 0..q  (pof/transitions.py:53-61)
  double f0 = 1.0, f1 = 1.0;
  for (int i = 2; i <= q; ++i) f0 *= i;
  for (int i = 2; i <= q - 1; ++i) f1 *= i;
  const double ah = fabs(h);
  *p0 = pow(ah, q + 0.5) / f0;
  *p1 = pow(ah, q - 0.5) / f1;
  return POF_OK;
}

int pof_linearize(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field, const void* params,
                  double h, const void* means, void* H, void* c, void* stream) {
  const Ops* ops = nullptr;
  int rc = check_common(dtype, n_steps, D, d, &ops);
  if (rc) return rc;
  if (field <= 0 || field >= FIELD_COUNT || field_dim(field) != d) return POF_ERR_FIELD;
  if (!params || !means || !H || !c) return POF_ERR_ARG;
  double p0, p1;
  rc = nordsieck_p01(D, d, h, &p0, &p1);
  if (rc) return rc;
  ops->linearize(n_steps, field, params, p0, p1, means, H, c, static_cast<cudaStream_t>(stream));
  return launch_status();
}

int pof_sequential_linear_filtsmooth(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, const void* x0_mean,
                                     const void* x0_chol, const void* F, const void* QL, int64_t ft_stride,
                                     const void* H, const void* c, const void* R, int64_t r_stride, int32_t smooth,
                                     void* out_mean, void* out_chol, double* out_scalars, void* stream) {
  const Ops* ops = nullptr;
  int rc = check_common(dtype, n_steps, D, d, &ops);
  if (rc) return rc;
  if (!x0_mean || !x0_chol || !F || !QL || !H || !c || !out_mean || !out_chol || !out_scalars) return POF_ERR_ARG;
  if (ft_stride != 0 && ft_stride != (int64_t)D * D) return POF_ERR_ARG;
  if (R && r_stride != 0 && r_stride != (int64_t)d * d) return POF_ERR_ARG;
  StepModel sm{F, QL, ft_stride, H, c, R, r_stride};
  ops->sequential(n_steps, sm, 0, nullptr, 0.0, 0.0, x0_mean, x0_chol, smooth, out_mean, out_chol, out_scalars,
                  static_cast<cudaStream_t>(stream));
  return launch_status();
}

int pof_sequential_eks(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field, const void* params,
                       double h, const void* x0_mean, const void* x0_chol, const void* F, const void* QL,
                       int64_t ft_stride, int32_t smooth, void* out_mean, void* out_chol, double* out_scalars,
                       void* stream) {
  const Ops* ops = nullptr;
  int rc = check_common(dtype, n_steps, D, d, &ops);
  if (rc) return rc;
  if (field <= 0 || field >= FIELD_COUNT || field_dim(field) != d) return POF_ERR_FIELD;
  if (!params || !x0_mean || !x0_chol || !F || !QL || !out_mean || !out_chol || !out_scalars) return POF_ERR_ARG;
  if (ft_stride != 0 && ft_stride != (int64_t)D * D) return POF_ERR_ARG;
  double p0, p1;
  rc = nordsieck_p01(D, d, h, &p0, &p1);
  if (rc) return rc;
  StepModel sm{F, QL, ft_stride, nullptr, nullptr, nullptr, 0};
  ops->sequential(n_steps, sm, field, params, p0, p1, x0_mean, x0_chol, smooth, out_mean, out_chol, out_scalars,
                  static_cast<cudaStream_t>(stream));
  return launch_status();
}

int pof_ieks_solve(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field, const void* params,
                   double h, const void* x0_mean, const void* x0_chol, const void* F, const void* QL, void* means,
                   void* chols, int64_t maxiters, int32_t calibrate, double* info, void* workspace,
                   size_t workspace_bytes, void* stream) {
  const Ops* ops = nullptr;
  int rc = check_common(dtype, n_steps, D, d, &ops);
  if (rc) return rc;
  if (field <= 0 || field >= FIELD_COUNT || field_dim(field) != d) return POF_ERR_FIELD;
  if (!params || !x0_mean || !x0_chol || !F || !QL || !means || !chols || !workspace || maxiters < 0)
    return POF_ERR_ARG;
  Plan p = plan_for(dtype, n_steps, D, d, true);
  if (workspace_bytes < p.total) return POF_ERR_WORKSPACE;
  double p0, p1;
  rc = nordsieck_p01(D, d, h, &p0, &p1);
  if (rc) return rc;
  char* w = aligned_ws(workspace);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t es = esz(dtype);
  double* scal = reinterpret_cast<double*>(w + p.scalars);
  void* Hb = w + p.H;
  void* cb = w + p.c;
  void* bufs[2] = {means, w + p.means2};
  k_init_scalars<<<1, 32, 0, st>>>(scal);
  StepModel sm{F, QL, 0, Hb, cb, nullptr, 0};
  int cur = 0;  // bufs[cur] holds the current states
  for (;;) {
    void* mold = bufs[cur];
    void* mnew = bufs[cur ^ 1];
    ops->linearize(n_steps, field, params, p0, p1, mold, Hb, cb, st);
    ops->filter(p, w, sm, x0_mean, x0_chol, mnew, chols, st);
    ops->smoother(p, w, F, QL, 0, mnew, chols, calibrate != 0, mold, st);
    {
      ProfScope ps(PK_CONTROL, st);
      k_ieks_control<<<1, 32, 0, st>>>(scal, maxiters);
    }
    rc = launch_status();
    if (rc) return rc;
    cur ^= 1;
    double cont = 0.0;
    cudaError_t e = cudaMemcpyAsync(&cont, scal + S_CONT, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    if (g_prof.on) prof_collect();
    if (cont == 0.0) break;
  }
  if (bufs[cur] != means) {
    cudaError_t e = cudaMemcpyAsync(means, bufs[cur], es * D * (n_steps + 1), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  if (calibrate) ops->scale_inplace(chols, (int64_t)D * D * (n_steps + 1), w + p.scale, st);
  if (info) k_copy_scalars<<<1, 32, 0, st>>>(scal, info, 1);
  return launch_status();
}

}  // extern "C"
