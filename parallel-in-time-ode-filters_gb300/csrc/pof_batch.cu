// C ABI of the batched IEKS solve (declared in include/pof.h): host loop,
// plan building and re-planning, CUDA-graph replay of the iteration.
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

std::vector<int64_t> step_offsets(int64_t B, const int64_t* n_steps) {
  std::vector<int64_t> so(B + 1);
  so[0] = 0;
  for (int64_t b = 0; b < B; ++b) so[b + 1] = so[b] + n_steps[b];
  return so;
}

// Workspace bytes of a batch: persistent part, then the level part of the
// plan over every problem (re-plans over fewer problems fit in it).
size_t batch_total(const BatchPersist& P, const BatchLevels& L) { return align_up(P.total) + L.total + 256; }

// The filter/smoother launches of one plan replayed from a CUDA graph of
// two iterations (the iterate buffers swap roles every iteration).
struct GraphPair {
  cudaGraphExec_t exec = nullptr;
  ~GraphPair() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
};

}  // namespace

extern "C" {

size_t pof_batch_workspace_bytes(int32_t dtype, int64_t B, const int64_t* n_steps, int32_t D, int32_t d,
                                 int32_t C0, int32_t Cg) {
  const BatchOps* ops = nullptr;
  if (check_batch(dtype, B, n_steps, D, d, &ops)) return 0;
  BatchPersist P = batch_persist(B, n_steps, D, d, dtype == POF_F32 ? 4 : 8);
  BatchShape sh = batch_shape(dtype, D, d, C0, Cg, P.n, ops);
  std::vector<int64_t> so = step_offsets(B, n_steps);
  std::vector<int32_t> all(B);
  for (int64_t b = 0; b < B; ++b) all[b] = (int32_t)b;
  BatchLevels L = batch_levels(sh, all, n_steps, so.data(), nullptr);
  if (L.cnt[L.nlev] != L.Ba) return 0;  // a problem too long for kMaxLevels levels
  return batch_total(P, L);
}

int pof_ieks_solve_batch(int32_t dtype, int64_t B, const int64_t* n_steps, int32_t D, int32_t d,
                         const int32_t* fields, const void* params, const double* h, const void* x0_mean,
                         const void* x0_chol, const void* F, const void* QL, void* means, void* chols,
                         int64_t maxiters, int32_t calibrate, int32_t C0, int32_t Cg, double* info, void* workspace,
                         size_t workspace_bytes, void* stream) {
  const BatchOps* ops = nullptr;
  int rc = check_batch(dtype, B, n_steps, D, d, &ops);
  if (rc) return rc;
  if (!fields || !h || !params || !x0_mean || !x0_chol || !F || !QL || !means || !chols || !workspace ||
      maxiters < 0)
    return POF_ERR_ARG;
  for (int64_t b = 0; b < B; ++b)
    if (fields[b] <= 0 || fields[b] >= FIELD_COUNT || field_dim(fields[b]) != d) return POF_ERR_FIELD;
  const int esz = dtype == POF_F32 ? 4 : 8;
  BatchPersist P = batch_persist(B, n_steps, D, d, esz);
  BatchShape sh = batch_shape(dtype, D, d, C0, Cg, P.n, ops);
  std::vector<int64_t> so = step_offsets(B, n_steps);
  std::vector<int32_t> active(B);
  for (int64_t b = 0; b < B; ++b) active[b] = (int32_t)b;
  std::vector<unsigned char> tab;
  BatchLevels L = batch_levels(sh, active, n_steps, so.data(), &tab);
  if (L.cnt[L.nlev] != L.Ba) return POF_ERR_ARG;  // a problem too long for kMaxLevels levels
  if (workspace_bytes < batch_total(P, L)) return POF_ERR_WORKSPACE;

  // persistent tables: step offsets, fields, Nordsieck scales
  std::vector<unsigned char> ptab(P.host_tab_bytes, 0);
  memcpy(ptab.data() + (P.so - P.host_tab), so.data(), sizeof(int64_t) * (B + 1));
  memcpy(ptab.data() + (P.fld - P.host_tab), fields, sizeof(int32_t) * B);
  double* p01 = reinterpret_cast<double*>(ptab.data() + (P.p01 - P.host_tab));
  for (int64_t b = 0; b < B; ++b)
    if (!nordsieck_scales(D, d, h[b], &p01[2 * b], &p01[2 * b + 1]) || !(h[b] != 0.0)) return POF_ERR_ARG;

  char* w = aligned_ws(workspace);
  char* lw = w + align_up(P.total);
  cudaStream_t us = static_cast<cudaStream_t>(stream);
  // own stream (graph capture needs one that is not the legacy default),
  // ordered after the caller's work and before the caller's later work
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  rc = cuda_status(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  if (rc) return rc;
  rc = cuda_status(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  if (!rc) rc = cuda_status(cudaEventRecord(ev, us));
  if (!rc) rc = cuda_status(cudaStreamWaitEvent(st, ev, 0));
  if (!rc) rc = cuda_status(cudaMemcpyAsync(w + P.host_tab, ptab.data(), P.host_tab_bytes, cudaMemcpyHostToDevice, st));
  if (!rc) rc = cuda_status(cudaMemsetAsync(w + P.pscal, 0, sizeof(double) * kBatchScalars * B, st));
  if (!rc) rc = cuda_status(cudaMemsetAsync(w + P.pscale, 0, sizeof(double) * B, st));
  if (!rc) rc = cuda_status(cudaMemsetAsync(w + P.frozen, 0, sizeof(int32_t) * B, st));

  int32_t* frozen = reinterpret_cast<int32_t*>(w + P.frozen);
  int32_t* nactive = reinterpret_cast<int32_t*>(w + P.nactive);
  void* bufs[2] = {means, w + P.means2};
  BatchRaw a{};
  a.params = params;
  a.x0m = x0_mean;
  a.x0L = x0_chol;
  a.F = F;
  a.QL = QL;
  a.H = w + P.H;
  a.c = w + P.c;
  a.selem = w + P.selem;
  a.chols = chols;
  a.pscal = reinterpret_cast<double*>(w + P.pscal);
  a.pscale = reinterpret_cast<double*>(w + P.pscale);
  a.frozen = frozen;
  a.nactive = nactive;
  a.maxiters = maxiters;
  a.rtol = 1e-6;  // crit's objective test (pof/convergence_criteria.py:4-13)
  a.atol = 1e-9;
  a.mrtol = 1e-13;
  a.matol = 1e-8;
  a.calibrate = calibrate != 0;
  a.team = sh.team;
  a.lw = lw;

  auto set_plan = [&](const BatchLevels& Lp) -> int {
    int r = cuda_status(cudaMemcpyAsync(lw, tab.data(), Lp.tab_bytes, cudaMemcpyHostToDevice, st));
    if (r) return r;
    a.L = &Lp;
    BView& v = a.v;
    v.so = reinterpret_cast<const int64_t*>(w + P.so);
    v.fld = reinterpret_cast<const int32_t*>(w + P.fld);
    v.p01 = reinterpret_cast<const double*>(w + P.p01);
    v.frozen = frozen;
    v.ap = reinterpret_cast<const int32_t*>(lw + Lp.ap);
    v.pc = reinterpret_cast<const int64_t*>(lw + Lp.pc);
    v.cs = reinterpret_cast<const int64_t*>(lw + Lp.cs);
    v.ce = reinterpret_cast<const int64_t*>(lw + Lp.ce);
    v.cp = reinterpret_cast<const int32_t*>(lw + Lp.cp);
    v.n = P.n;
    v.n1 = Lp.cnt[1];
    v.Ba = Lp.Ba;
    v.C0 = Lp.C0max;
    return POF_OK;
  };
  if (!rc) rc = set_plan(L);

  const bool use_graph = !prof_on() && env_int("POF_BATCH_NO_GRAPH") == 0;
  GraphPair gp;
  auto capture = [&]() -> int {
    gp.reset();
    cudaGraph_t g = nullptr;
    int r = cuda_status(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    if (r) return r;
    ops->iteration(a, bufs[0], bufs[1], st);
    ops->iteration(a, bufs[1], bufs[0], st);
    r = cuda_status(cudaStreamEndCapture(st, &g));
    if (r) return r;
    r = cuda_status(cudaGraphInstantiate(&gp.exec, g, 0));
    cudaGraphDestroy(g);
    return r;
  };
  if (!rc && use_graph) rc = capture();

  std::vector<int32_t> hfrozen(B);
  int32_t hactive = 0;
  // every problem stops after at most maxiters + 1 iterations; two per round
  const int64_t max_rounds = maxiters / 2 + 2;
  for (int64_t round = 0; !rc && round < max_rounds; ++round) {
    if (use_graph) {
      rc = cuda_status(cudaGraphLaunch(gp.exec, st));
    } else {
      ops->iteration(a, bufs[0], bufs[1], st);
      ops->iteration(a, bufs[1], bufs[0], st);
      rc = launch_status();
    }
    if (!rc) rc = cuda_status(cudaMemcpyAsync(&hactive, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
    if (rc) break;
    if (prof_on()) prof_flush();
    if (hactive == 0) break;
    // drop converged problems from the plan once they hold half its steps
    rc = cuda_status(cudaMemcpyAsync(hfrozen.data(), frozen, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, st));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
    if (rc) break;
    std::vector<int32_t> still;
    int64_t steps = 0;
    for (int32_t b : active)
      if (!hfrozen[b]) {
        still.push_back(b);
        steps += n_steps[b];
      }
    if (!still.empty() && 2 * steps < L.steps) {
      active.swap(still);
      L = batch_levels(sh, active, n_steps, so.data(), &tab);
      rc = set_plan(L);
      if (!rc) rc = cuda_status(cudaStreamSynchronize(st));  // tab is host memory of this frame
      if (!rc && use_graph) rc = capture();
    }
  }
  if (!rc) {
    ops->finish(B, reinterpret_cast<const int64_t*>(w + P.so), a.pscal, a.pscale, a.calibrate, means, bufs[1], chols,
                info, st);
    rc = launch_status();
  }
  // the caller's stream waits for this work
  if (cudaEventRecord(ev, st) == cudaSuccess) cudaStreamWaitEvent(us, ev, 0);
  cudaEventDestroy(ev);
  cudaStreamDestroy(st);
  return rc;
}

}  // extern "C"
