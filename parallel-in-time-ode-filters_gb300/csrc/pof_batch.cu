// C ABI of the batched IEKS solves (declared in include/pof.h): plan
// building and re-planning, the device-resident loops (float64, and the
// float32 phase of the mixed-precision form) replayed from CUDA graphs.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/pof.h"
#include "pof_batch.cuh"

using namespace pof;

namespace {

int env_int(const char* name) {
  const char* v = getenv(name);
  return v ? atoi(v) : 0;
}

// Chunk length, group size and team sizes of a batch.  POF_BATCH_C0,
// POF_BATCH_CG and POF_BATCH_TEAM_WIDE=1 override the defaults (tuning).
BatchShape batch_shape(int dtype, int D, int d, int C0, int Cg, int64_t total_steps, const BatchOps* ops) {
  BatchShape sh;
  sh.D = D;
  sh.DY = d;
  sh.esz = dtype == POF_F32 ? 4 : 8;
  sh.team = env_int("POF_BATCH_TEAM_WIDE") ? ops->tsw : ops->tsn;
  sh.team_up = ops->tsw;
  if (C0 <= 0) C0 = env_int("POF_BATCH_C0");
  sh.C0 = C0 > 0 ? C0 : batch_pick_c0(total_steps, sh.team);
  if (Cg <= 1) Cg = env_int("POF_BATCH_CG");
  sh.Cg = Cg > 1 ? Cg : 2;
  return sh;
}

int check_batch(int32_t dtype, int64_t B, const int64_t* n_steps, int32_t D, int32_t d, const BatchOps** ops) {
  if (dtype != POF_F64 && dtype != POF_F32) return POF_ERR_DTYPE;
  if (B < 1 || B > (int64_t)0x7fffffff || !n_steps || D < 1 || d < 1 || D % d) return POF_ERR_ARG;
  for (int64_t b = 0; b < B; ++b)
    if (n_steps[b] < 1) return POF_ERR_ARG;
  *ops = find_batch_shape(dtype, D, d);
  return *ops ? POF_OK : POF_ERR_SHAPE;
}

int check_fields(int64_t B, int32_t d, const int32_t* fields, const double* h) {
  if (!fields || !h) return POF_ERR_ARG;
  for (int64_t b = 0; b < B; ++b)
    if (fields[b] <= 0 || fields[b] >= FIELD_COUNT || field_dim(fields[b]) != d) return POF_ERR_FIELD;
  return POF_OK;
}

struct GraphExec {
  cudaGraphExec_t exec = nullptr;
  ~GraphExec() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
};

// One batch in one element type: its workspace regions, its plan over the
// problems still running, and the arguments of its launches.
struct BatchCtx {
  int64_t B = 0;
  const int64_t* n_steps = nullptr;
  const BatchOps* ops = nullptr;
  BatchShape sh;
  BatchPersist P;
  BatchLevels L;
  std::vector<int64_t> gb;  // first grid point of each problem
  std::vector<int32_t> active;
  std::vector<unsigned char> tab;
  char* w = nullptr;   // persistent part
  char* lw = nullptr;  // level part
  BatchRaw a{};
  GraphExec graph;

  // Sizes only (no device pointers yet).
  int init(int32_t dtype, int64_t B_, const int64_t* ns, int32_t D, int32_t d, int32_t C0, int32_t Cg) {
    int rc = check_batch(dtype, B_, ns, D, d, &ops);
    if (rc) return rc;
    B = B_;
    n_steps = ns;
    gb.assign(B, 0);
    int64_t G = 0, steps = 0;
    for (int64_t b = 0; b < B; ++b) {
      gb[b] = G;
      G += ns[b] + 1;
      steps += ns[b];
    }
    P = batch_persist(B, G, D, d, dtype == POF_F32 ? 4 : 8);
    sh = batch_shape(dtype, D, d, C0, Cg, steps, ops);
    active.resize(B);
    for (int64_t b = 0; b < B; ++b) active[b] = (int32_t)b;
    L = batch_levels(sh, active, ns, gb.data(), nullptr, &tab);
    if (L.cnt[L.nlev] != L.Ba) return POF_ERR_ARG;  // a problem too long for kMaxLevels levels
    return POF_OK;
  }
  size_t bytes() const { return align_up(P.total) + align_up(L.total); }

  // Persistent tables (step offsets, fields, Nordsieck scales) to the device,
  // per-problem state cleared.
  int place(char* base, const int32_t* fields, const double* h, cudaStream_t st) {
    w = base;
    lw = base + align_up(P.total);
    std::vector<unsigned char> ptab(P.host_tab_bytes, 0);
    memcpy(ptab.data() + (P.gb - P.host_tab), gb.data(), sizeof(int64_t) * B);
    memcpy(ptab.data() + (P.ns - P.host_tab), n_steps, sizeof(int64_t) * B);
    memcpy(ptab.data() + (P.fld - P.host_tab), fields, sizeof(int32_t) * B);
    double* p01 = reinterpret_cast<double*>(ptab.data() + (P.p01 - P.host_tab));
    for (int64_t b = 0; b < B; ++b)
      if (!(h[b] != 0.0) || !nordsieck_scales(sh.D, sh.DY, h[b], &p01[2 * b], &p01[2 * b + 1])) return POF_ERR_ARG;
    int rc = cuda_status(cudaMemcpyAsync(w + P.host_tab, ptab.data(), P.host_tab_bytes, cudaMemcpyHostToDevice, st));
    if (!rc) rc = cuda_status(cudaMemsetAsync(w + P.pscal, 0, sizeof(double) * kBatchScalars * B, st));
    if (!rc) rc = cuda_status(cudaMemsetAsync(w + P.pscale, 0, sizeof(double) * B, st));
    if (!rc) rc = cuda_status(cudaMemsetAsync(w + P.frozen, 0, sizeof(int32_t) * B, st));
    // ptab is host memory of this frame: the copy must have left it
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
    a.H = w + P.H;
    a.c = w + P.c;
    a.selem = w + P.selem;
    a.pscal = reinterpret_cast<double*>(w + P.pscal);
    a.pscale = reinterpret_cast<double*>(w + P.pscale);
    a.frozen = reinterpret_cast<int32_t*>(w + P.frozen);
    a.nactive = reinterpret_cast<int32_t*>(w + P.nactive);
    a.lw = lw;
    a.team = sh.team;
    a.rtol = 1e-6;  // crit (pof/convergence_criteria.py:4-13)
    a.atol = 1e-9;
    a.mrtol = 1e-13;
    a.matol = 1e-8;
    if (!rc) rc = set_plan(st);
    return rc;
  }

  // Upload the level tables of L and point the launches at them.
  int set_plan(cudaStream_t st) {
    int rc = cuda_status(cudaMemcpyAsync(lw, tab.data(), L.tab_bytes, cudaMemcpyHostToDevice, st));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
    a.L = &L;
    BView& v = a.v;
    v.gb = reinterpret_cast<const int64_t*>(w + P.gb);
    v.ns = reinterpret_cast<const int64_t*>(w + P.ns);
    v.fld = reinterpret_cast<const int32_t*>(w + P.fld);
    v.rtol = nullptr;
    v.maxit = nullptr;
    v.cancel = nullptr;
    v.p01 = reinterpret_cast<const double*>(w + P.p01);
    v.frozen = a.frozen;
    v.ap = reinterpret_cast<const int32_t*>(lw + L.ap);
    v.pc = reinterpret_cast<const int64_t*>(lw + L.pc);
    v.cs = reinterpret_cast<const int64_t*>(lw + L.cs);
    v.ce = reinterpret_cast<const int64_t*>(lw + L.ce);
    v.cp = reinterpret_cast<const int32_t*>(lw + L.cp);
    v.n = P.G;
    v.nb = B;
    v.n1 = L.cnt[1];
    v.Ba = L.Ba;
    v.C0 = L.C0max;
    return rc;
  }

  // Re-plan over the problems not yet frozen once the frozen ones hold half
  // the plan's steps.  Sets *replanned.
  int maybe_replan(cudaStream_t st, bool* replanned) {
    *replanned = false;
    std::vector<int32_t> hfrozen(B);
    int rc = cuda_status(cudaMemcpyAsync(hfrozen.data(), a.frozen, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, st));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
    if (rc) return rc;
    std::vector<int32_t> still;
    int64_t steps = 0;
    for (int32_t b : active)
      if (!hfrozen[b]) {
        still.push_back(b);
        steps += n_steps[b];
      }
    if (still.empty() || 2 * steps >= L.steps) return POF_OK;
    active.swap(still);
    L = batch_levels(sh, active, n_steps, gb.data(), nullptr, &tab);
    *replanned = true;
    return set_plan(st);
  }

  template <typename F>
  int capture(cudaStream_t st, F&& body) {
    graph.reset();
    cudaGraph_t g = nullptr;
    int rc = cuda_status(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    if (rc) return rc;
    body();
    rc = cuda_status(cudaStreamEndCapture(st, &g));
    if (rc) return rc;
    rc = cuda_status(cudaGraphInstantiate(&graph.exec, g, 0));
    cudaGraphDestroy(g);
    return rc;
  }
};

bool graphs_on() { return !prof_on() && env_int("POF_BATCH_NO_GRAPH") == 0; }

int read_count(const int32_t* dev, int32_t* host, cudaStream_t st) {
  int rc = cuda_status(cudaMemcpyAsync(host, dev, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
  if (!rc && prof_on()) prof_flush();
  return rc;
}

// The float64 IEKS loop (pof/solver.py:36-57 per problem) from the iterate
// in bufs[0]; two iterations per round (the buffers swap roles), one host
// read per round.  The latest iterate of problem b is in bufs[iterations_b % 2].
int loop_f64(BatchCtx& c, void* bufs[2], int64_t maxiters, cudaStream_t st) {
  const bool use_graph = graphs_on();
  auto body = [&]() {
    c.ops->iteration(c.a, bufs[0], bufs[1], st);
    c.ops->iteration(c.a, bufs[1], bufs[0], st);
  };
  int rc = use_graph ? c.capture(st, body) : POF_OK;
  int32_t hactive = 0;
  const int64_t max_rounds = maxiters / 2 + 2;  // every problem stops by iteration maxiters + 1
  for (int64_t round = 0; !rc && round < max_rounds; ++round) {
    if (use_graph) {
      rc = cuda_status(cudaGraphLaunch(c.graph.exec, st));
    } else {
      body();
      rc = launch_status();
    }
    if (!rc) rc = read_count(c.a.nactive, &hactive, st);
    if (rc || hactive == 0) break;
    bool replanned = false;
    rc = c.maybe_replan(st, &replanned);
    if (!rc && replanned && use_graph) rc = c.capture(st, body);
  }
  return rc;
}

// Own stream for the batch (graph capture needs one that is not the legacy
// default), ordered after the caller's work; the caller's later work waits
// for it (StreamJoin::done).
struct StreamJoin {
  cudaStream_t us = nullptr, st = nullptr;
  cudaEvent_t ev = nullptr;
  int open(void* stream) {
    us = static_cast<cudaStream_t>(stream);
    int rc = cuda_status(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    if (!rc) rc = cuda_status(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    if (!rc) rc = cuda_status(cudaEventRecord(ev, us));
    if (!rc) rc = cuda_status(cudaStreamWaitEvent(st, ev, 0));
    return rc;
  }
  ~StreamJoin() {
    if (ev && st && cudaEventRecord(ev, st) == cudaSuccess) cudaStreamWaitEvent(us, ev, 0);
    if (ev) cudaEventDestroy(ev);
    if (st) cudaStreamDestroy(st);
  }
};

// Workspace of the mixed-precision batch after the float64 and float32
// contexts: float32 chols, x0, F, QL, the input trajectories (float64) and
// the per-problem float32-phase state.
struct MixedExtras {
  size_t chols32, x0m32, x0L32, F32, QL32, keep, mst, total;
};
MixedExtras mixed_extras(const BatchCtx& c) {
  MixedExtras e;
  const int D = c.sh.D;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  e.chols32 = take(sizeof(float) * D * D * c.P.G);
  e.x0m32 = take(sizeof(float) * D * c.B);
  e.x0L32 = take(sizeof(float) * D * D * c.B);
  e.F32 = take(sizeof(float) * D * D);
  e.QL32 = take(sizeof(float) * D * D);
  e.keep = take(sizeof(double) * D * c.P.G);
  e.mst = take(sizeof(double) * M_COUNT * c.B);
  e.total = off;
  return e;
}

unsigned g256(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

extern "C" {

size_t pof_batch_workspace_bytes(int32_t dtype, int64_t B, const int64_t* n_steps, int32_t D, int32_t d,
                                 int32_t C0, int32_t Cg) {
  BatchCtx c;
  if (c.init(dtype, B, n_steps, D, d, C0, Cg)) return 0;
  return c.bytes() + 256;
}

int pof_ieks_solve_batch(int32_t dtype, int64_t B, const int64_t* n_steps, int32_t D, int32_t d,
                         const int32_t* fields, const void* params, const double* h, const void* x0_mean,
                         const void* x0_chol, const void* F, const void* QL, void* means, void* chols,
                         int64_t maxiters, int32_t calibrate, int32_t C0, int32_t Cg, double* info, void* workspace,
                         size_t workspace_bytes, void* stream) {
  BatchCtx c;
  int rc = c.init(dtype, B, n_steps, D, d, C0, Cg);
  if (rc) return rc;
  rc = check_fields(B, d, fields, h);
  if (rc) return rc;
  if (!params || !x0_mean || !x0_chol || !F || !QL || !means || !chols || !workspace || maxiters < 0)
    return POF_ERR_ARG;
  if (workspace_bytes < c.bytes() + 256) return POF_ERR_WORKSPACE;
  for (int64_t b = 0; b < B; ++b)
    if (!(h[b] != 0.0)) return POF_ERR_ARG;
  StreamJoin sj;
  rc = sj.open(stream);
  if (rc) return rc;
  cudaStream_t st = sj.st;
  rc = c.place(aligned_ws(workspace), fields, h, st);
  if (rc) return rc;
  c.a.params = params;
  c.a.x0m = x0_mean;
  c.a.x0L = x0_chol;
  c.a.F = F;
  c.a.QL = QL;
  c.a.chols = chols;
  c.a.maxiters = maxiters;
  c.a.calibrate = calibrate != 0;
  void* bufs[2] = {means, c.w + c.P.means2};
  rc = loop_f64(c, bufs, maxiters, st);
  if (rc) return rc;
  c.ops->finish(B, c.a.v.gb, c.a.v.ns, c.a.pscal, c.a.pscale, c.a.calibrate, means, bufs[1], chols, info, st);
  return launch_status();
}

size_t pof_batch_mixed_workspace_bytes(int64_t B, const int64_t* n_steps, int32_t D, int32_t d, int32_t C0,
                                       int32_t Cg) {
  BatchCtx c64, c32;
  if (c64.init(POF_F64, B, n_steps, D, d, C0, Cg) || c32.init(POF_F32, B, n_steps, D, d, C0, Cg)) return 0;
  return c64.bytes() + c32.bytes() + mixed_extras(c32).total + 256;
}

int pof_ieks_solve_batch_mixed(int64_t B, const int64_t* n_steps, int32_t D, int32_t d, const int32_t* fields,
                               const double* params, const double* h, const double* x0_mean, const double* x0_chol,
                               const double* F, const double* QL, double* means, double* chols, int64_t maxiters_f32,
                               double rtol_f32, double settle_f32, int64_t maxiters, int32_t calibrate, int32_t C0,
                               int32_t Cg, double* info, double* info_f32, void* workspace, size_t workspace_bytes,
                               void* stream) {
  BatchCtx c64, c32;
  int rc = c64.init(POF_F64, B, n_steps, D, d, C0, Cg);
  if (!rc) rc = c32.init(POF_F32, B, n_steps, D, d, C0, Cg);
  if (rc) return rc;
  rc = check_fields(B, d, fields, h);
  if (rc) return rc;
  if (!params || !x0_mean || !x0_chol || !F || !QL || !means || !chols || !workspace || maxiters < 0 ||
      maxiters_f32 < 0 || !(rtol_f32 > 0) || !(settle_f32 > 0))
    return POF_ERR_ARG;
  const MixedExtras ex = mixed_extras(c32);
  if (workspace_bytes < c64.bytes() + c32.bytes() + ex.total + 256) return POF_ERR_WORKSPACE;
  for (int64_t b = 0; b < B; ++b)
    if (!(h[b] != 0.0)) return POF_ERR_ARG;
  StreamJoin sj;
  rc = sj.open(stream);
  if (rc) return rc;
  cudaStream_t st = sj.st;
  char* base = aligned_ws(workspace);
  char* x = base + c64.bytes() + c32.bytes();
  rc = c64.place(base, fields, h, st);
  if (!rc) rc = c32.place(base + c64.bytes(), fields, h, st);
  if (rc) return rc;
  const int64_t G = c64.P.G;
  float* chols32 = reinterpret_cast<float*>(x + ex.chols32);
  float* x0m32 = reinterpret_cast<float*>(x + ex.x0m32);
  float* x0L32 = reinterpret_cast<float*>(x + ex.x0L32);
  float* F32 = reinterpret_cast<float*>(x + ex.F32);
  float* QL32 = reinterpret_cast<float*>(x + ex.QL32);
  double* keep = reinterpret_cast<double*>(x + ex.keep);
  double* mst = reinterpret_cast<double*>(x + ex.mst);
  float* m32 = reinterpret_cast<float*>(c32.w + c32.P.means2);
  kb_d2f<<<g256(B * D), 256, 0, st>>>(x0_mean, x0m32, B * D);
  kb_d2f<<<g256(B * D * D), 256, 0, st>>>(x0_chol, x0L32, B * D * D);
  kb_d2f<<<g256(D * D), 256, 0, st>>>(F, F32, D * D);
  kb_d2f<<<g256(D * D), 256, 0, st>>>(QL, QL32, D * D);
  kb_init_mixed<<<g256(B * M_COUNT), 256, 0, st>>>(mst, B);
  rc = cuda_status(cudaMemcpyAsync(keep, means, sizeof(double) * D * G, cudaMemcpyDeviceToDevice, st));
  if (rc) return rc;

  // float32 phase: float64 linearization at the float64 iterate, float32
  // filter/smoother, the change judged in float64 (pof_ieks_solve_mixed's
  // rules, per problem); c32's frozen flags mark the problems done with it
  BatchRaw& a = c32.a;
  a.params = nullptr;
  a.x0m = x0m32;
  a.x0L = x0L32;
  a.F = F32;
  a.QL = QL32;
  a.chols = chols32;
  a.calibrate = false;
  a.maxiters = maxiters_f32;
  if (maxiters_f32 > 0) {
    const bool use_graph = graphs_on();
    auto body = [&]() {
      cudaMemsetAsync(a.nactive, 0, sizeof(int32_t), st);
      c32.ops->lin_mixed(a.v, params, means, static_cast<float*>(a.H), static_cast<float*>(a.c), st);
      c32.ops->filtsmooth(a, nullptr, m32, st);
      c32.ops->ychange(a.v, m32, means, mst, st);
      kb_ctl32<<<g256(a.v.Ba), 256, 0, st>>>(a.v, mst, a.frozen, maxiters_f32, rtol_f32, settle_f32, a.nactive);
      c32.ops->accept(a.v, m32, means, mst, st);
    };
    rc = use_graph ? c32.capture(st, body) : POF_OK;
    int32_t hactive = 0;
    for (int64_t it = 0; !rc && it < maxiters_f32; ++it) {
      if (use_graph) {
        rc = cuda_status(cudaGraphLaunch(c32.graph.exec, st));
      } else {
        body();
        rc = launch_status();
      }
      if (!rc) rc = read_count(a.nactive, &hactive, st);
      if (rc || hactive == 0) break;
      bool replanned = false;
      rc = c32.maybe_replan(st, &replanned);
      if (!rc && replanned && use_graph) rc = c32.capture(st, body);
    }
    if (rc) return rc;
    c32.ops->revert(B, c32.a.v.gb, c32.a.v.ns, mst, rtol_f32, keep, means, st);
  }

  // float64 polish: the reference loop per problem from the kept iterates
  c64.a.params = params;
  c64.a.x0m = x0_mean;
  c64.a.x0L = x0_chol;
  c64.a.F = F;
  c64.a.QL = QL;
  c64.a.chols = chols;
  c64.a.maxiters = maxiters;
  c64.a.calibrate = calibrate != 0;
  void* bufs[2] = {means, c64.w + c64.P.means2};
  rc = loop_f64(c64, bufs, maxiters, st);
  if (rc) return rc;
  c64.ops->finish(B, c64.a.v.gb, c64.a.v.ns, c64.a.pscal, c64.a.pscale, c64.a.calibrate, means, bufs[1], chols, info,
                  st);
  if (info_f32) {
    static_assert(M_BEST == M_IT + 1, "info_f32 copies (iterations, best change) as one pair");
    rc = cuda_status(cudaMemcpy2DAsync(info_f32, 2 * sizeof(double), mst + M_IT, sizeof(double) * M_COUNT,
                                       2 * sizeof(double), B, cudaMemcpyDeviceToDevice, st));
    if (rc) return rc;
  }
  return launch_status();
}

}  // extern "C"
