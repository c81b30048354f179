// C ABI of libpof.so (declared in include/pof.h).
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/pof.h"
#include "pof_dense.h"
#include "pof_table.cuh"

using namespace pof;

namespace {
thread_local std::string g_cuda_error;
}  // namespace

namespace pof {
// Status of a CUDA runtime call; the message is kept for pof_last_cuda_error.
int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return POF_OK;
  g_cuda_error = cudaGetErrorString(e);
  return POF_ERR_CUDA;
}

int launch_status() { return cuda_status(cudaGetLastError()); }

char* aligned_ws(void* ws) {
  uintptr_t a = reinterpret_cast<uintptr_t>(ws);
  a = (a + 255) & ~uintptr_t(255);
  return reinterpret_cast<char*>(a);
}

int wide_lane_limit() {
  const char* v = getenv("POF_WIDE_LANES");
  return v ? atoi(v) : 16384;
}
}  // namespace pof

namespace {

const Ops* find_ops(int dtype, int D, int DY) {
  if (dtype != POF_F64 && dtype != POF_F32) return nullptr;
  if (DY < 1 || D < 1) return nullptr;
  return find_shape(dtype, D, DY);
}

int esz(int dtype) { return dtype == POF_F32 ? 4 : 8; }

// Optional overrides (tuning): POF_C0, POF_CG chunk sizes; POF_TEAM_WIDE_L0=1
// runs level 0 with the wide team kernels; POF_KS the largest top level
// scanned in parallel (ks_limit: 0, the default, always the binary tree up to
// kTop elements; -1 the lane-count rule).  In the float32 iterations of the
// mixed-precision solve the parallel top also settles higher (Van der Pol
// mu = 10, q = 4, N = 4096: smallest float32 change 2.0e-3 with a 512-element
// parallel top, 6.5e-4 with the tree).
int env_int(const char* name, int dflt = 0) {
  const char* v = getenv(name);
  return v ? atoi(v) : dflt;
}

Plan plan_for(int dtype, int64_t n, int D, int DY, bool solver) {
  return make_plan(n, D, DY, esz(dtype), solver, env_int("POF_C0"), env_int("POF_CG"),
                   env_int("POF_TEAM_WIDE_L0") != 0, env_int("POF_KS", 0));
}

// The sequential filter/smoother as a plan: one level-0 chunk spanning all
// n steps, so one team runs the square-root Kalman filter and the RTS
// smoother step after step (the level-0 kernels' recursion, from x0 and
// from the terminal state), nothing above it.
Plan sequential_plan(int dtype, int64_t n, int D, int DY) {
  const int C0 = n < (int64_t)0x7fffffff ? (int)n : 0x7fffffff;
  return make_plan(n, D, DY, esz(dtype), true, C0, 0, false, 0);
}

int check_common(int dtype, int64_t n, int D, int DY, const Ops** ops) {
  if (dtype != POF_F64 && dtype != POF_F32) return POF_ERR_DTYPE;
  if (n < 1 || D < 1 || DY < 1) return POF_ERR_ARG;
  *ops = find_ops(dtype, D, DY);
  if (!*ops) return POF_ERR_SHAPE;
  return POF_OK;
}

// The filter's scalars are reported through the same block layout.
void report_scalars(const Plan& p, char* ws, double* out, cudaStream_t st) {
  if (out) k_copy_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(ws + p.scalars), out, 0);
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
void prof_flush() { prof_collect(); }
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

#ifdef POF_CHECKS
namespace pof {
__device__ unsigned long long pof_check_line = 0;
}
#endif

extern "C" {

int pof_checks_compiled(void) {
#ifdef POF_CHECKS
  return 1;
#else
  return 0;
#endif
}

int pof_checks_read(uint64_t* line_out, int32_t reset) {
  if (!line_out) return POF_ERR_ARG;
  *line_out = 0;
#ifdef POF_CHECKS
  unsigned long long v = 0;
  int rc = cuda_status(cudaMemcpyFromSymbol(&v, pof::pof_check_line, sizeof(v)));
  if (rc) return rc;
  *line_out = v;
  if (reset) {
    const unsigned long long zero = 0;
    rc = cuda_status(cudaMemcpyToSymbol(pof::pof_check_line, &zero, sizeof(zero)));
    if (rc) return rc;
  }
#else
  (void)reset;
#endif
  return POF_OK;
}

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

// rcp_nr / rsqrt_nr on an array (diagnostics: their accuracy against IEEE
// division and square root is checked by the tests).
__global__ void k_recip_check(int64_t n, const double* __restrict__ x, double* __restrict__ r, double* __restrict__ q) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  r[i] = rcp_nr(x[i]);
  q[i] = x[i] > 0.0 ? rsqrt_nr(x[i]) : 0.0;
}

int pof_recip_check(int64_t n, const double* x, double* rcp_out, double* rsqrt_out, void* stream) {
  if (n < 1 || !x || !rcp_out || !rsqrt_out) return POF_ERR_ARG;
  k_recip_check<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, x, rcp_out, rsqrt_out);
  return launch_status();
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
    case POF_ERR_BUSY: return "no free request slot or memory (retry later)";
    default: return "unknown status";
  }
}

const char* pof_last_cuda_error(void) { return g_cuda_error.c_str(); }

int pof_version(void) { return 2; }

int pof_shape_supported(int32_t D, int32_t d) { return find_ops(POF_F64, D, d) != nullptr ? 1 : 0; }

// Shapes the small-D tables do not compile, with D >= dense::kMinD, run on
// the dense path (pof_dense.cu).
static bool dense_shape(int dtype, int D, int d) {
  return (dtype == POF_F64 || dtype == POF_F32) && D >= dense::kMinD && d >= 1 && !find_ops(dtype, D, d);
}

size_t pof_filtsmooth_workspace_bytes(int32_t dtype, int64_t n_steps, int32_t D, int32_t d) {
  if (n_steps < 1 || D < 1) return 0;
  if (dense_shape(dtype, D, d)) return dense::workspace_bytes(dtype, 1, n_steps, D, d, 0);
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
  if (rc == POF_ERR_SHAPE && dense_shape(dtype, D, d))
    return pof_dense_linear_filtsmooth(which, dtype, n, D, d, x0m, x0L, F, QL, fts, H, c, R, rs, om, oL, osc, 0, ws,
                                       wsb, stream);
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
  if (!ops && D >= dense::kMinD)
    return pof_dense_linear_filtsmooth(POF_DENSE_SMOOTHING, dtype, n_steps, D, 1, filt_mean, filt_chol, F, QL,
                                       ft_stride, nullptr, nullptr, nullptr, 0, out_mean, out_chol, out_scalars, 0,
                                       workspace, workspace_bytes, stream);
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

size_t pof_dense_workspace_bytes(int32_t dtype, int32_t which, int64_t n_steps, int32_t D, int32_t d,
                                 int32_t chunks) {
  if (dtype != POF_F64 && dtype != POF_F32) return 0;
  if (which < POF_DENSE_FILTER || which > POF_DENSE_SMOOTHING || d < 1) return 0;
  return dense::workspace_bytes(dtype, which, n_steps, D, d, chunks);
}

int pof_dense_linear_filtsmooth(int32_t which, int32_t dtype, int64_t n_steps, int32_t D, int32_t d,
                                const void* x0_mean, const void* x0_chol, const void* F, const void* QL,
                                int64_t ft_stride, const void* H, const void* c, const void* R, int64_t r_stride,
                                void* out_mean, void* out_chol, double* out_scalars, int32_t chunks, void* workspace,
                                size_t workspace_bytes, void* stream) {
  if (dtype != POF_F64 && dtype != POF_F32) return POF_ERR_DTYPE;
  if (which < POF_DENSE_FILTER || which > POF_DENSE_SMOOTHING) return POF_ERR_ARG;
  if (n_steps < 1 || D < 1 || d < 1 || chunks < 0) return POF_ERR_ARG;
  if (n_steps > 0x7fffffffLL || (int64_t)D * (D + d) > 0x7fffffffLL) return POF_ERR_ARG;
  if (!x0_mean || !x0_chol || !F || !QL || !out_mean || !out_chol || !workspace) return POF_ERR_ARG;
  if (which != POF_DENSE_SMOOTHING && (!H || !c)) return POF_ERR_ARG;
  if (ft_stride != 0 && ft_stride != (int64_t)D * D) return POF_ERR_ARG;
  if (R && r_stride != 0 && r_stride != (int64_t)d * d) return POF_ERR_ARG;
  if (workspace_bytes < dense::workspace_bytes(dtype, which, n_steps, D, d, chunks)) return POF_ERR_WORKSPACE;
  return dense::filtsmooth(which, dtype, n_steps, D, d, x0_mean, x0_chol, F, QL, ft_stride, H, c, R, r_stride,
                           out_mean, out_chol, out_scalars, chunks, workspace, workspace_bytes,
                           static_cast<cudaStream_t>(stream));
}

static int nordsieck_p01(int D, int d, double h, double* p0, double* p1) {
  return nordsieck_scales(D, d, h, p0, p1) ? POF_OK : POF_ERR_ARG;
}

int pof_linearize(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field, const void* params,
                  double h, const void* means, void* H, void* c, void* stream) {
  if (field == FIELD_FHN_RD) {
    // any shape: d = 2 x cells, D = d (q + 1)
    if (dtype != POF_F64 && dtype != POF_F32) return POF_ERR_DTYPE;
    if (n_steps < 1 || D < 1 || d < 2 || n_steps > 0x7fffffffLL) return POF_ERR_ARG;
    if (d % 2) return POF_ERR_FIELD;
    if (!params || !means || !H || !c) return POF_ERR_ARG;
    double p0, p1;
    int rc = nordsieck_p01(D, d, h, &p0, &p1);
    if (rc) return rc;
    return dense::linearize(dtype, n_steps, D, d, field, params, p0, p1, means, H, c,
                            static_cast<cudaStream_t>(stream));
  }
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

}  // extern "C"

namespace {

__global__ void k_d2f(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}
__global__ void k_f2d(const float* __restrict__ in, double* __restrict__ out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (double)in[i];
}

struct Loop {
  const Ops* ops;
  const Plan* p;
  char* w;           // aligned workspace of this plan
  int field;
  const void* params;
  double p0, p1;
  const void* x0m;
  const void* x0L;
  const void* F;
  const void* QL;
  void* means;       // in: initial trajectory, out: result
  void* chols;
  size_t esz;
  int64_t maxiters;
  bool calibrate;
  double rtol, atol;  // objective test of crit
};

// The IEKS loop as one CUDA graph: a while node whose body is one iteration
// -- linearize at the iterate in l.means, filter and smooth into the second
// buffer, loop control (k_ieks_control_graph sets the while condition),
// copy the new iterate back into l.means -- so the whole loop runs on the
// device without a host round trip per iteration.  The instantiated graph
// is kept for the next call with the same arguments (one per host thread).
struct GraphLoopKey {
  const Ops* ops;
  int64_t n, maxiters;
  int D, DY, C0, Cg, nlev, field, dev;
  bool ks, calibrate;
  const void *params, *x0m, *x0L, *F, *QL, *means, *chols;
  char* w;
  double p0, p1, rtol, atol;
  bool same(const GraphLoopKey& o) const {
    return ops == o.ops && n == o.n && maxiters == o.maxiters && D == o.D && DY == o.DY && C0 == o.C0 &&
           Cg == o.Cg && nlev == o.nlev && field == o.field && dev == o.dev && ks == o.ks &&
           calibrate == o.calibrate && params == o.params && x0m == o.x0m && x0L == o.x0L && F == o.F &&
           QL == o.QL && means == o.means && chols == o.chols && w == o.w && p0 == o.p0 && p1 == o.p1 &&
           rtol == o.rtol && atol == o.atol;
  }
};

// No destructor: an instantiated graph kept at process exit is released
// with the context (a CUDA call during static destruction may find the
// runtime gone).
struct GraphLoopCache {
  bool valid = false;
  GraphLoopKey key{};
  cudaGraphExec_t exec = nullptr;
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    valid = false;
  }
};
thread_local GraphLoopCache g_loop_graph;

// The graph's while loop ends by itself after maxiters + 1 iterations at the
// latest; loops allowed more than kGraphMaxIters iterations are launched from
// the host instead, so a process can always be interrupted between launches.
constexpr int64_t kGraphMaxIters = 100000;

bool loop_graphs_on(int64_t maxiters) {
  return !g_prof.on && env_int("POF_SOLVE_NO_GRAPH") == 0 && maxiters <= kGraphMaxIters;
}

int build_loop_graph(const Loop& l, cudaStream_t st, cudaGraphExec_t* out) {
  const Plan& p = *l.p;
  char* w = l.w;
  double* scal = reinterpret_cast<double*>(w + p.scalars);
  void* Hb = w + p.H;
  void* cb = w + p.c;
  void* mnew = w + p.means2;
  StepModel sm{l.F, l.QL, 0, Hb, cb, nullptr, 0};
  cudaGraph_t g = nullptr;
  int rc = cuda_status(cudaGraphCreate(&g, 0));
  if (rc) return rc;
  cudaGraphConditionalHandle handle;
  rc = cuda_status(cudaGraphConditionalHandleCreate(&handle, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (!rc) rc = cuda_status(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
  if (!rc) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    // a private stream for the capture, so nothing else of the caller's
    // stream joins the body
    cudaStream_t cs = nullptr;
    rc = cuda_status(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    if (!rc) rc = cuda_status(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal));
    if (!rc) {
      l.ops->linearize(p.n, l.field, l.params, l.p0, l.p1, l.means, Hb, cb, cs);
      l.ops->filter(p, w, sm, l.x0m, l.x0L, mnew, l.chols, cs);
      l.ops->smoother(p, w, l.F, l.QL, 0, mnew, l.chols, l.calibrate, l.means, cs);
      k_ieks_control_graph<<<1, 32, 0, cs>>>(scal, l.maxiters, l.rtol, l.atol, handle);
      cudaMemcpyAsync(l.means, mnew, l.esz * p.D * (p.n + 1), cudaMemcpyDeviceToDevice, cs);
      cudaGraph_t captured = nullptr;
      const int rc2 = cuda_status(cudaStreamEndCapture(cs, &captured));
      rc = launch_status();
      if (!rc) rc = rc2;
    }
    if (cs) cudaStreamDestroy(cs);
  }
  if (!rc) rc = cuda_status(cudaGraphInstantiate(out, g, 0));
  cudaGraphDestroy(g);
  (void)st;
  return rc;
}

int ieks_loop_graph(const Loop& l, cudaStream_t st) {
  const Plan& p = *l.p;
  int dev = 0;
  int rc = cuda_status(cudaGetDevice(&dev));
  if (rc) return rc;
  GraphLoopKey key{l.ops, p.n, l.maxiters, p.D, p.DY, p.C0, p.Cg, p.nlev, l.field, dev, p.ks, l.calibrate,
                   l.params, l.x0m, l.x0L, l.F, l.QL, l.means, l.chols, l.w, l.p0, l.p1, l.rtol, l.atol};
  GraphLoopCache& c = g_loop_graph;
  if (!(c.valid && c.key.same(key))) {
    c.reset();
    rc = build_loop_graph(l, st, &c.exec);
    if (rc) {
      c.reset();
      return rc;
    }
    c.key = key;
    c.valid = true;
  }
  k_init_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(l.w + p.scalars));
  rc = launch_status();
  if (!rc) rc = cuda_status(cudaGraphLaunch(c.exec, st));
  return rc;
}

// The IEKS loop of pof/solver.py:36-57 on the device: as one CUDA graph
// (ieks_loop_graph), or -- with the event profiler on, or POF_SOLVE_NO_GRAPH
// set -- launched from the host with one read of the loop condition per
// iteration.  Leaves the result in l.means and the scalars (nll, obj, ssq,
// iterations, status) in the plan's scalar block.
int ieks_loop(const Loop& l, cudaStream_t st) {
  if (loop_graphs_on(l.maxiters)) return ieks_loop_graph(l, st);
  const Plan& p = *l.p;
  char* w = l.w;
  double* scal = reinterpret_cast<double*>(w + p.scalars);
  void* Hb = w + p.H;
  void* cb = w + p.c;
  void* bufs[2] = {l.means, w + p.means2};
  k_init_scalars<<<1, 32, 0, st>>>(scal);
  StepModel sm{l.F, l.QL, 0, Hb, cb, nullptr, 0};
  int cur = 0;  // bufs[cur] holds the current states
  for (;;) {
    void* mold = bufs[cur];
    void* mnew = bufs[cur ^ 1];
    l.ops->linearize(p.n, l.field, l.params, l.p0, l.p1, mold, Hb, cb, st);
    l.ops->filter(p, w, sm, l.x0m, l.x0L, mnew, l.chols, st);
    l.ops->smoother(p, w, l.F, l.QL, 0, mnew, l.chols, l.calibrate, mold, st);
    {
      ProfScope ps(PK_CONTROL, st);
      k_ieks_control<<<1, 32, 0, st>>>(scal, l.maxiters, l.rtol, l.atol);
    }
    int rc = launch_status();
    if (rc) return rc;
    cur ^= 1;
    double cont = 0.0;
    cudaError_t e = cudaMemcpyAsync(&cont, scal + S_CONT, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    if (g_prof.on) prof_collect();
    if (cont == 0.0) break;
  }
  if (bufs[cur] != l.means) {
    cudaError_t e = cudaMemcpyAsync(l.means, bufs[cur], l.esz * p.D * (p.n + 1), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return POF_OK;
}

// Workspace of the mixed-precision solve: the float64 solver plan, the
// float32 filter/smoother plan, float copies of the problem, and a float64
// candidate trajectory.
struct MixedLayout {
  Plan p64, p32;
  size_t off32, fmeans, fchols, fx0m, fx0L, fF, fQL, fH, fc, cand, keep, red, total;
};

MixedLayout mixed_layout(int64_t n, int D, int d) {
  MixedLayout m;
  m.p64 = plan_for(POF_F64, n, D, d, true);
  m.p32 = plan_for(POF_F32, n, D, d, false);
  size_t off = align_up(m.p64.total);
  m.off32 = off;
  off = align_up(off + m.p32.total);
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  m.fmeans = take(sizeof(float) * D * (n + 1));
  m.fchols = take(sizeof(float) * D * D * (n + 1));
  m.fx0m = take(sizeof(float) * D);
  m.fx0L = take(sizeof(float) * D * D);
  m.fF = take(sizeof(float) * D * D);
  m.fQL = take(sizeof(float) * D * D);
  m.fH = take(sizeof(float) * d * D * n);
  m.fc = take(sizeof(float) * d * n);
  m.cand = take(sizeof(double) * D * (n + 1));
  m.keep = take(sizeof(double) * D * (n + 1));
  m.red = take(sizeof(unsigned long long) * 4);
  m.total = off + 256;
  return m;
}

// Rows of a noiseless observation model can be scaled freely (0 = H x + c
// is the same constraint as 0 = (H x + c) / s): normalize each row of
// (H, c) and convert to float32, which keeps the float32 filter clear of the
// huge Jacobians of early IEKS iterates.
__global__ void k_rows_to_f32(const double* __restrict__ H, const double* __restrict__ c, float* __restrict__ Hf,
                              float* __restrict__ cf, int64_t rows, int D) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double s = 0.0;
  for (int k = 0; k < D; ++k) s = fma(H[r * D + k], H[r * D + k], s);
  const double inv = s > 0.0 ? 1.0 / sqrt(s) : 1.0;
  for (int k = 0; k < D; ++k) Hf[r * D + k] = (float)(H[r * D + k] * inv);
  cf[r] = (float)(c[r] * inv);
}

// max |y_new - y_old|, max |y_old| over the projected states y = p0 m[i(q+1)]
// (bit patterns of non-negative doubles order like the values, so atomicMax
// on them is exact and order-independent), and a non-finite flag.
__global__ void k_ychange(const double* __restrict__ mnew, const double* __restrict__ mold, int64_t N, int D, int d,
                          double p0, unsigned long long* __restrict__ red) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int Q1 = D / d;
  double dy = 0.0, ay = 0.0;
  bool bad = false;
  if (idx < N * d) {
    const int64_t k = idx / d;
    const int i = (int)(idx % d);
    const double a = mnew[k * D + i * Q1], b = mold[k * D + i * Q1];
    bad = !isfinite(a);
    dy = fabs(p0 * (a - b));
    ay = fabs(p0 * b);
  }
  for (int o = 16; o > 0; o >>= 1) {
    dy = fmax(dy, __shfl_xor_sync(0xffffffffu, dy, o));
    ay = fmax(ay, __shfl_xor_sync(0xffffffffu, ay, o));
    bad = bad || __shfl_xor_sync(0xffffffffu, (int)bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicOr(&red[2], 1ull);
    if (isfinite(dy)) atomicMax(&red[0], (unsigned long long)__double_as_longlong(dy));
    if (isfinite(ay)) atomicMax(&red[1], (unsigned long long)__double_as_longlong(ay));
  }
}

unsigned g1d(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

extern "C" {

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
  Loop l{ops, &p, w, field, params, p0, p1, x0_mean, x0_chol, F, QL, means, chols, (size_t)esz(dtype),
         maxiters, calibrate != 0, 1e-6, 1e-9};
  rc = ieks_loop(l, st);
  if (rc) return rc;
  if (calibrate) ops->scale_inplace(chols, (int64_t)D * D * (n_steps + 1), w + p.scale, st);
  if (info) k_copy_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(w + p.scalars), info, 1);
  return launch_status();
}

size_t pof_ieks_sequential_workspace_bytes(int32_t dtype, int64_t n_steps, int32_t D, int32_t d) {
  if (n_steps < 1 || D < 1) return 0;
  return sequential_plan(dtype, n_steps, D, d).total;
}

int pof_ieks_solve_sequential(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field,
                              const void* params, double h, const void* x0_mean, const void* x0_chol, const void* F,
                              const void* QL, void* means, void* chols, int64_t maxiters, int32_t calibrate,
                              double* info, void* workspace, size_t workspace_bytes, void* stream) {
  const Ops* ops = nullptr;
  int rc = check_common(dtype, n_steps, D, d, &ops);
  if (rc) return rc;
  if (field <= 0 || field >= FIELD_COUNT || field_dim(field) != d) return POF_ERR_FIELD;
  if (!params || !x0_mean || !x0_chol || !F || !QL || !means || !chols || !workspace || maxiters < 0)
    return POF_ERR_ARG;
  Plan p = sequential_plan(dtype, n_steps, D, d);
  if (workspace_bytes < p.total) return POF_ERR_WORKSPACE;
  double p0, p1;
  rc = nordsieck_p01(D, d, h, &p0, &p1);
  if (rc) return rc;
  char* w = aligned_ws(workspace);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Loop l{ops, &p, w, field, params, p0, p1, x0_mean, x0_chol, F, QL, means, chols, (size_t)esz(dtype),
         maxiters, calibrate != 0, 1e-6, 1e-9};
  rc = ieks_loop(l, st);
  if (rc) return rc;
  if (calibrate) ops->scale_inplace(chols, (int64_t)D * D * (n_steps + 1), w + p.scale, st);
  if (info) k_copy_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(w + p.scalars), info, 1);
  return launch_status();
}

size_t pof_ieks_mixed_workspace_bytes(int64_t n_steps, int32_t D, int32_t d) {
  if (n_steps < 1 || D < 1) return 0;
  return mixed_layout(n_steps, D, d).total;
}

int pof_ieks_solve_mixed(int64_t n_steps, int32_t D, int32_t d, int32_t field, const double* params, double h,
                         const double* x0_mean, const double* x0_chol, const double* F, const double* QL,
                         double* means, double* chols, int64_t maxiters_f32, double rtol_f32, double settle_f32,
                         int64_t maxiters,
                         int32_t calibrate, double* info, void* workspace, size_t workspace_bytes, void* stream) {
  const Ops* ops64 = nullptr;
  const Ops* ops32 = nullptr;
  int rc = check_common(POF_F64, n_steps, D, d, &ops64);
  if (rc) return rc;
  rc = check_common(POF_F32, n_steps, D, d, &ops32);
  if (rc) return rc;
  if (field <= 0 || field >= FIELD_COUNT || field_dim(field) != d) return POF_ERR_FIELD;
  if (!params || !x0_mean || !x0_chol || !F || !QL || !means || !chols || !workspace || maxiters < 0 ||
      maxiters_f32 < 0 || !(rtol_f32 > 0) || !(settle_f32 > 0))
    return POF_ERR_ARG;
  MixedLayout m = mixed_layout(n_steps, D, d);
  if (workspace_bytes < m.total) return POF_ERR_WORKSPACE;
  double p0, p1;
  rc = nordsieck_p01(D, d, h, &p0, &p1);
  if (rc) return rc;
  char* w = aligned_ws(workspace);
  char* w32 = w + m.off32;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int64_t N = n_steps + 1;
  const int64_t NM = (int64_t)D * N;
  float* fm = reinterpret_cast<float*>(w + m.fmeans);
  float* fL = reinterpret_cast<float*>(w + m.fchols);
  float* fx0m = reinterpret_cast<float*>(w + m.fx0m);
  float* fx0L = reinterpret_cast<float*>(w + m.fx0L);
  float* fF = reinterpret_cast<float*>(w + m.fF);
  float* fQL = reinterpret_cast<float*>(w + m.fQL);
  float* fH = reinterpret_cast<float*>(w + m.fH);
  float* fc = reinterpret_cast<float*>(w + m.fc);
  double* cand = reinterpret_cast<double*>(w + m.cand);
  double* keep = reinterpret_cast<double*>(w + m.keep);
  unsigned long long* red = reinterpret_cast<unsigned long long*>(w + m.red);
  double* H64 = reinterpret_cast<double*>(w + m.p64.H);
  double* c64 = reinterpret_cast<double*>(w + m.p64.c);
  k_d2f<<<1, 256, 0, st>>>(x0_mean, fx0m, D);
  k_d2f<<<g1d(D * D), 256, 0, st>>>(x0_chol, fx0L, D * D);
  k_d2f<<<g1d(D * D), 256, 0, st>>>(F, fF, D * D);
  k_d2f<<<g1d(D * D), 256, 0, st>>>(QL, fQL, D * D);
  k_init_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(w32 + m.p32.scalars));
  StepModel sm32{fF, fQL, 0, fH, fc, nullptr, 0};
  // float32 phase: linearize in float64, filter/smooth in float32, measure
  // each step's change in float64
  int64_t it32 = 0;
  double prev = 1e300, best = 1e300;
  int worse = 0;
  const double settle = settle_f32;
  {
    cudaError_t e = cudaMemcpyAsync(keep, means, sizeof(double) * NM, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  while (it32 < maxiters_f32) {
    ops64->linearize(n_steps, field, params, p0, p1, means, H64, c64, st);
    k_rows_to_f32<<<g1d(n_steps * d), 256, 0, st>>>(H64, c64, fH, fc, n_steps * d, D);
    ops32->filter(m.p32, w32, sm32, fx0m, fx0L, fm, fL, st);
    ops32->smoother(m.p32, w32, fF, fQL, 0, fm, fL, false, nullptr, st);
    k_f2d<<<g1d(NM), 256, 0, st>>>(fm, cand, NM);
    cudaError_t e = cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 4, st);
    if (e != cudaSuccess) return cuda_status(e);
    k_ychange<<<g1d(N * d), 256, 0, st>>>(cand, means, N, D, d, p0, red);
    rc = launch_status();
    if (rc) return rc;
    unsigned long long hred[3];
    e = cudaMemcpyAsync(hred, red, sizeof(hred), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    double dy, ay;
    memcpy(&dy, &hred[0], sizeof(double));
    memcpy(&ay, &hred[1], sizeof(double));
    if (hred[2] != 0) break;  // non-finite float32 iterate: keep the last float64 one
    ++it32;
    e = cudaMemcpyAsync(means, cand, sizeof(double) * NM, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
    const double rel = ay > 0.0 ? dy / ay : dy;
    best = rel < best ? rel : best;
    if (rel < rtol_f32) break;       // converged as far as float32 goes
    // non-shrinking changes count once the change is below `settle` (the
    // IEKS's first iterations from a crude initial trajectory are not
    // monotone); HUGE_VAL counts every one
    worse = (rel >= prev && best < settle) ? worse + 1 : (rel >= prev ? worse : 0);
    if (worse >= 3) break;           // float32 stopped helping
    prev = rel;
  }
  // a float32 phase that never came near convergence (an ill-conditioned
  // smoother in float32) is discarded: the polish starts from the input
  if (it32 > 0 && !(best < 100.0 * rtol_f32)) {
    cudaError_t e = cudaMemcpyAsync(means, keep, sizeof(double) * NM, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(e);
    it32 = 0;
  }
  // float64 polish: the reference loop from the last accepted trajectory
  Loop l64{ops64, &m.p64, w, field, params, p0, p1, x0_mean, x0_chol, F, QL, means, chols, sizeof(double),
           maxiters, calibrate != 0, 1e-6, 1e-9};
  rc = ieks_loop(l64, st);
  if (rc) return rc;
  if (calibrate) ops64->scale_inplace(chols, (int64_t)D * D * N, w + m.p64.scale, st);
  if (info) {
    k_copy_scalars<<<1, 32, 0, st>>>(reinterpret_cast<double*>(w + m.p64.scalars), info, 1);
    const double extra[2] = {(double)it32, best};
    cudaError_t e = cudaMemcpyAsync(info + POF_I_COUNT, extra, sizeof(extra), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return launch_status();
}

}  // extern "C"
