// Continuous-batching IEKS engine (declared in include/pof.h): requests of
// one state shape (D, d) are admitted into a device-resident arena while
// others are iterating, every tick runs one IEKS iteration over all admitted
// and unfinished requests (the batched, per-problem segmented scan of
// pof_batch.cuh), and finished requests leave the plan and free their
// memory.  A request's result depends only on its own inputs: its chunk
// length comes from its own step count (serve_c0) and no arithmetic mixes
// two requests, so it is the same alone and in any mix.
#include <cuda_runtime.h>
#include <string.h>

#include <vector>

#include "../../include/pof.h"
#include "pof_arena.h"
#include "pof_batch.cuh"

using namespace pof;

namespace {

// Steps per level-0 chunk of a request with n steps (a function of n only).
int serve_c0(int64_t n) {
  int64_t c = 4;
  while (c < 64 && c * 2 * 256 <= n) c *= 2;
  return (int)c;
}

// Per-request block uploaded at admission and scattered by ks_admit.
struct AdmitBlock {
  int64_t gb, ns, maxit;
  int32_t fld, pad;
  double p01[2], params[4], rtol;
};

struct Extras {
  size_t means, chols, params, x0m, x0L, rtol, maxit, F, QL, admit, row, total;
};

Extras serve_extras(int D, int64_t maxB, int64_t maxG) {
  Extras e;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  e.means = take(sizeof(double) * D * maxG);
  e.chols = take(sizeof(double) * D * D * maxG);
  e.params = take(sizeof(double) * 4 * maxB);
  e.x0m = take(sizeof(double) * D * maxB);
  e.x0L = take(sizeof(double) * D * D * maxB);
  e.rtol = take(sizeof(double) * maxB);
  e.maxit = take(sizeof(int64_t) * maxB);
  e.F = take(sizeof(double) * D * D);
  e.QL = take(sizeof(double) * D * D);
  e.admit = take(sizeof(AdmitBlock));
  e.row = take(sizeof(double) * (D + D + D * D));  // init row, x0 mean, x0 chol of one request
  e.total = off;
  return e;
}

// Writes one request's slot from its uploaded block and fills its grid
// range of the current iterate buffer with the initial row.
__global__ void ks_admit(int32_t b, const AdmitBlock* __restrict__ blk, const double* __restrict__ rows, int D,
                         int64_t* gb, int64_t* ns, int32_t* fld, double* p01, double* params, double* rtol,
                         int64_t* maxit, double* x0m, double* x0L, double* pscal, double* pscale, int32_t* frozen,
                         double* means) {
  const AdmitBlock& a = *blk;
  const int64_t N = a.ns + 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * D; i += (int64_t)gridDim.x * blockDim.x)
    means[a.gb * D + i] = rows[i % D];
  if (blockIdx.x != 0) return;
  for (int i = threadIdx.x; i < D; i += blockDim.x) x0m[(int64_t)b * D + i] = rows[D + i];
  for (int i = threadIdx.x; i < D * D; i += blockDim.x) x0L[(int64_t)b * D * D + i] = rows[2 * D + i];
  for (int i = threadIdx.x; i < kBatchScalars; i += blockDim.x) pscal[(int64_t)kBatchScalars * b + i] = 0.0;
  if (threadIdx.x == 0) {
    gb[b] = a.gb;
    ns[b] = a.ns;
    fld[b] = a.fld;
    p01[2 * b] = a.p01[0];
    p01[2 * b + 1] = a.p01[1];
    for (int k = 0; k < 4; ++k) params[4 * b + k] = a.params[k];
    rtol[b] = a.rtol;
    maxit[b] = a.maxit;
    pscale[b] = 0.0;
    frozen[b] = 0;
  }
}

// A finished request's result: the latest iterate (buffer by the parity of
// its iteration count), the calibrated chol (pof/solver.py:66-69) and
// info = (iterations, nll, obj, sigma^2, status).
__global__ void ks_fetch(int32_t b, int parity0, const int64_t* __restrict__ gb, const int64_t* __restrict__ ns,
                         const double* __restrict__ m0, const double* __restrict__ m1,
                         const double* __restrict__ chols, const double* __restrict__ pscal,
                         const double* __restrict__ pscale, int calibrate, int D, double* __restrict__ out_m,
                         double* __restrict__ out_L, double* __restrict__ info) {
  const double* sc = pscal + (int64_t)kBatchScalars * b;
  const long long it = (long long)sc[S_ITER];
  const double* m = ((parity0 ^ (int)(it & 1)) == 0) ? m0 : m1;
  const int64_t g0 = gb[b], N = ns[b] + 1;
  const double s = calibrate ? pscale[b] : 1.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * D; i += stride) out_m[i] = m[g0 * D + i];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * D * D; i += stride)
    out_L[i] = chols[g0 * D * D + i] * s;
  if (info && blockIdx.x == 0 && threadIdx.x == 0) {
    info[POF_I_ITERATIONS] = sc[S_ITER];
    info[POF_I_NLL] = sc[S_NLL];
    info[POF_I_OBJ] = sc[S_OBJ];
    info[POF_I_SSQ] = sc[S_SSQ];
    info[POF_I_STATUS] = sc[S_STATUS];
  }
}

struct Slot {
  bool used = false, finished = false;
  bool phase32 = false;  // in its float32 phase (mixed-precision engine)
  int64_t g0 = 0, ns = 0;
  int parity0 = 0;
};

// Workspace of a mixed-precision engine after the float64 engine's: the
// float32 batch state (persistent part and a level part of the same cap),
// float32 chols and copies of x0, F, QL, the float64 iterate of the requests
// in their float32 phase (mcur), their input trajectories (keep, for the
// discard rule) and the per-request float32-phase state (mst).
struct MixedServe {
  BatchPersist P32;
  size_t p32, lw32, chols32, x0m32, x0L32, F32, QL32, mcur, keep, mst, total;
};

MixedServe mixed_serve_layout(int D, int d, int64_t maxB, int64_t maxG, size_t level_cap) {
  MixedServe m;
  m.P32 = batch_persist(maxB, maxG, D, d, 4);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align_up(off + bytes);
    return o;
  };
  m.p32 = take(m.P32.total);
  m.lw32 = take(level_cap);
  m.chols32 = take(sizeof(float) * D * D * maxG);
  m.x0m32 = take(sizeof(float) * D * maxB);
  m.x0L32 = take(sizeof(float) * D * D * maxB);
  m.F32 = take(sizeof(float) * D * D);
  m.QL32 = take(sizeof(float) * D * D);
  m.mcur = take(sizeof(double) * D * maxG);
  m.keep = take(sizeof(double) * D * maxG);
  m.mst = take(sizeof(double) * M_COUNT * maxB);
  m.total = off;
  return m;
}

// A request of a mixed-precision engine starts in its float32 phase: its
// float64 iterate (mcur) and the copy the discard rule returns to (keep)
// get the initial rows, x0 goes to float32, its float32-phase state is
// reset, and the float64 plan skips it (frozen) until the phase ends.
__global__ void ks_admit_mixed(int32_t b, const AdmitBlock* __restrict__ blk, const double* __restrict__ rows, int D,
                               double* mcur, double* keep, float* x0m32, float* x0L32, double* mst, int32_t* done32,
                               int32_t* frozen64) {
  const AdmitBlock& a = *blk;
  const int64_t N = a.ns + 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N * D; i += (int64_t)gridDim.x * blockDim.x) {
    mcur[a.gb * D + i] = rows[i % D];
    keep[a.gb * D + i] = rows[i % D];
  }
  if (blockIdx.x != 0) return;
  for (int i = threadIdx.x; i < D; i += blockDim.x) x0m32[(int64_t)b * D + i] = (float)rows[D + i];
  for (int i = threadIdx.x; i < D * D; i += blockDim.x) x0L32[(int64_t)b * D * D + i] = (float)rows[2 * D + i];
  for (int f = threadIdx.x; f < M_COUNT; f += blockDim.x)
    mst[(int64_t)M_COUNT * b + f] = (f == M_BEST || f == M_PREV) ? 1e300 : 0.0;
  if (threadIdx.x == 0) {
    done32[b] = 0;
    frozen64[b] = 1;
  }
}

static __global__ void ks_d2f(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)in[i];
}

static __global__ void ks_mixed_info(const double* __restrict__ mst, int32_t b, double* __restrict__ out) {
  if (threadIdx.x == 0) {
    out[0] = mst[(int64_t)M_COUNT * b + M_IT];
    out[1] = mst[(int64_t)M_COUNT * b + M_BEST];
  }
}

}  // namespace

struct pof_server {
  int D = 0, d = 0;
  int64_t maxB = 0, maxG = 0;
  size_t level_cap = 0;
  bool calibrate = true;
  const BatchOps* ops = nullptr;
  BatchShape sh;
  BatchPersist P;
  Extras X;
  char* w = nullptr;   // persistent part
  char* lw = nullptr;  // level part
  char* xw = nullptr;  // extras
  cudaStream_t st = nullptr;
  BatchRaw a{};
  BatchLevels L;
  std::vector<unsigned char> tab;
  std::vector<int32_t> active;
  std::vector<Slot> slots;
  std::vector<int64_t> h_gb, h_ns, done;
  std::vector<int32_t> h_c0, h_frozen;
  Arena arena;
  void* bufs[2] = {nullptr, nullptr};
  // Cancel flags, one per slot, in mapped pinned host memory: the host sets
  // them (pof_server_cancel) and kb_control reads them at every tick.
  volatile int32_t* h_cancel = nullptr;
  int32_t* d_cancel = nullptr;
  int cur = 0;  // bufs[cur] holds the current iterates
  bool dirty = true;
  int64_t ticks = 0;
  // mixed precision: requests start with float32 IEKS iterations (the rules
  // of pof_ieks_solve_batch_mixed's float32 phase), then go on in float64
  bool mixed = false;
  int64_t maxiters_f32 = 0;
  double rtol_f32 = 1e-5, settle_f32 = 1e300;
  const BatchOps* ops32 = nullptr;
  BatchShape sh32;
  MixedServe M;
  char* mw = nullptr;  // mixed part of the workspace
  BatchRaw a32{};
  BatchLevels L32;
  std::vector<unsigned char> tab32;
  std::vector<int32_t> active32, h_done32;

  double* mcur() const { return reinterpret_cast<double*>(mw + M.mcur); }
  double* mst() const { return reinterpret_cast<double*>(mw + M.mst); }

  int replan32() {
    active32.clear();
    for (int64_t b = 0; b < maxB; ++b)
      if (slots[b].used && !slots[b].finished && slots[b].phase32) active32.push_back((int32_t)b);
    if (active32.empty()) return POF_OK;
    L32 = batch_levels(sh32, active32, h_ns.data(), h_gb.data(), h_c0.data(), &tab32);
    char* lw32 = mw + M.lw32;
    int rc = cuda_status(cudaMemcpyAsync(lw32, tab32.data(), L32.tab_bytes, cudaMemcpyHostToDevice, st));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
    a32.L = &L32;
    BView& v = a32.v;
    v.ap = reinterpret_cast<const int32_t*>(lw32 + L32.ap);
    v.pc = reinterpret_cast<const int64_t*>(lw32 + L32.pc);
    v.cs = reinterpret_cast<const int64_t*>(lw32 + L32.cs);
    v.ce = reinterpret_cast<const int64_t*>(lw32 + L32.ce);
    v.cp = reinterpret_cast<const int32_t*>(lw32 + L32.cp);
    v.n1 = L32.cnt[1];
    v.Ba = L32.Ba;
    v.C0 = L32.C0max;
    return rc;
  }

  // One float32 iteration of every request in its float32 phase: float64
  // linearization at its float64 iterate, float32 filter/smoother, the
  // change judged in float64, the phase's stopping rules, kept candidates
  // into the float64 iterate.
  void tick32() {
    BatchRaw& a = a32;
    cudaMemsetAsync(a.nactive, 0, sizeof(int32_t), st);
    ops32->lin_mixed(a.v, static_cast<const double*>(this->a.params), mcur(), static_cast<float*>(a.H),
                     static_cast<float*>(a.c), st);
    float* m32 = reinterpret_cast<float*>(mw + M.p32 + M.P32.means2);
    ops32->filtsmooth(a, nullptr, m32, st);
    ops32->ychange(a.v, m32, mcur(), mst(), st);
    kb_ctl32<<<(unsigned)((a.v.Ba + 255) / 256), 256, 0, st>>>(a.v, mst(), a.frozen, maxiters_f32, rtol_f32,
                                                                settle_f32, a.nactive);
    ops32->accept(a.v, m32, mcur(), mst(), st);
  }

  int replan() {
    active.clear();
    for (int64_t b = 0; b < maxB; ++b)
      if (slots[b].used && !slots[b].finished && !slots[b].phase32) active.push_back((int32_t)b);
    dirty = false;
    if (mixed) {
      const int rc = replan32();
      if (rc) return rc;
    }
    if (active.empty()) return POF_OK;
    L = batch_levels(sh, active, h_ns.data(), h_gb.data(), h_c0.data(), &tab);
    int rc = cuda_status(cudaMemcpyAsync(lw, tab.data(), L.tab_bytes, cudaMemcpyHostToDevice, st));
    if (!rc) rc = cuda_status(cudaStreamSynchronize(st));
    a.L = &L;
    BView& v = a.v;
    v.ap = reinterpret_cast<const int32_t*>(lw + L.ap);
    v.pc = reinterpret_cast<const int64_t*>(lw + L.pc);
    v.cs = reinterpret_cast<const int64_t*>(lw + L.cs);
    v.ce = reinterpret_cast<const int64_t*>(lw + L.ce);
    v.cp = reinterpret_cast<const int32_t*>(lw + L.cp);
    v.n1 = L.cnt[1];
    v.Ba = L.Ba;
    v.C0 = L.C0max;
    return rc;
  }
};

extern "C" {

size_t pof_server_workspace_bytes(int32_t D, int32_t d, int64_t max_requests, int64_t max_points,
                                  size_t level_bytes) {
  if (!find_batch_shape(POF_F64, D, d) || max_requests < 1 || max_points < 2) return 0;
  BatchPersist P = batch_persist(max_requests, max_points, D, d, 8);
  return align_up(P.total) + align_up(level_bytes) + serve_extras(D, max_requests, max_points).total + 256;
}

size_t pof_server_mixed_workspace_bytes(int32_t D, int32_t d, int64_t max_requests, int64_t max_points,
                                        size_t level_bytes) {
  const size_t base = pof_server_workspace_bytes(D, d, max_requests, max_points, level_bytes);
  if (!base || !find_batch_shape(POF_F32, D, d)) return 0;
  return base + mixed_serve_layout(D, d, max_requests, max_points, align_up(level_bytes)).total;
}

}  // extern "C"

namespace {

int server_create(int32_t D, int32_t d, int64_t max_requests, int64_t max_points, size_t level_bytes,
                  const double* F, const double* QL, int32_t calibrate, bool mixed, int64_t maxiters_f32,
                  double rtol_f32, double settle_f32, void* workspace, size_t workspace_bytes, pof_server** out) {
  if (!out || !F || !QL || !workspace) return POF_ERR_ARG;
  *out = nullptr;
  const BatchOps* ops = find_batch_shape(POF_F64, D, d);
  if (!ops) return POF_ERR_SHAPE;
  const BatchOps* ops32 = mixed ? find_batch_shape(POF_F32, D, d) : nullptr;
  if (mixed && !ops32) return POF_ERR_SHAPE;
  if (max_requests < 1 || max_requests > (int64_t)0x7fffffff || max_points < 2) return POF_ERR_ARG;
  if (mixed && (maxiters_f32 < 0 || !(rtol_f32 > 0) || !(settle_f32 > 0))) return POF_ERR_ARG;
  const size_t need = mixed ? pof_server_mixed_workspace_bytes(D, d, max_requests, max_points, level_bytes)
                            : pof_server_workspace_bytes(D, d, max_requests, max_points, level_bytes);
  if (workspace_bytes < need) return POF_ERR_WORKSPACE;
  pof_server* s = new pof_server();
  s->D = D;
  s->d = d;
  s->maxB = max_requests;
  s->maxG = max_points;
  s->level_cap = align_up(level_bytes);
  s->calibrate = calibrate != 0;
  s->ops = ops;
  s->sh.D = D;
  s->sh.DY = d;
  s->sh.esz = 8;
  s->sh.team = ops->tsn;
  s->sh.team_up = ops->tsw;
  s->sh.C0 = 4;
  s->sh.Cg = 2;
  s->P = batch_persist(max_requests, max_points, D, d, 8);
  s->X = serve_extras(D, max_requests, max_points);
  s->w = aligned_ws(workspace);
  s->lw = s->w + align_up(s->P.total);
  s->xw = s->lw + s->level_cap;
  s->slots.assign(max_requests, Slot());
  s->h_gb.assign(max_requests, 0);
  s->h_ns.assign(max_requests, 1);
  s->h_c0.assign(max_requests, 4);
  s->h_frozen.assign(max_requests, 1);
  s->arena.init(max_points);
  int rc = cuda_status(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking));
  if (!rc) {
    void* hc = nullptr;
    rc = cuda_status(cudaHostAlloc(&hc, sizeof(int32_t) * max_requests, cudaHostAllocMapped));
    if (!rc) {
      memset(hc, 0, sizeof(int32_t) * max_requests);
      s->h_cancel = static_cast<volatile int32_t*>(hc);
      void* dc = nullptr;
      rc = cuda_status(cudaHostGetDevicePointer(&dc, hc, 0));
      s->d_cancel = static_cast<int32_t*>(dc);
    }
  }
  const BatchPersist& P = s->P;
  char* w = s->w;
  if (!rc) rc = cuda_status(cudaMemsetAsync(w + P.frozen, 0xff, sizeof(int32_t) * max_requests, s->st));
  if (!rc) rc = cuda_status(cudaMemcpyAsync(s->xw + s->X.F, F, sizeof(double) * D * D, cudaMemcpyDeviceToDevice, s->st));
  if (!rc)
    rc = cuda_status(cudaMemcpyAsync(s->xw + s->X.QL, QL, sizeof(double) * D * D, cudaMemcpyDeviceToDevice, s->st));
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s->st));
  if (rc) {
    if (s->st) cudaStreamDestroy(s->st);
    if (s->h_cancel) cudaFreeHost(const_cast<int32_t*>(s->h_cancel));
    delete s;
    return rc;
  }
  BatchRaw& a = s->a;
  char* x = s->xw;
  a.params = x + s->X.params;
  a.x0m = x + s->X.x0m;
  a.x0L = x + s->X.x0L;
  a.F = x + s->X.F;
  a.QL = x + s->X.QL;
  a.H = w + P.H;
  a.c = w + P.c;
  a.selem = w + P.selem;
  a.chols = x + s->X.chols;
  a.pscal = reinterpret_cast<double*>(w + P.pscal);
  a.pscale = reinterpret_cast<double*>(w + P.pscale);
  a.frozen = reinterpret_cast<int32_t*>(w + P.frozen);
  a.nactive = reinterpret_cast<int32_t*>(w + P.nactive);
  a.maxiters = 0;  // per request (v.maxit)
  a.rtol = 1e-6;   // per request (v.rtol)
  a.atol = 1e-9;
  a.mrtol = 1e-13;
  a.matol = 1e-8;
  a.calibrate = s->calibrate;
  a.team = s->sh.team;
  a.lw = s->lw;
  BView& v = a.v;
  v.gb = reinterpret_cast<const int64_t*>(w + P.gb);
  v.ns = reinterpret_cast<const int64_t*>(w + P.ns);
  v.fld = reinterpret_cast<const int32_t*>(w + P.fld);
  v.p01 = reinterpret_cast<const double*>(w + P.p01);
  v.frozen = a.frozen;
  v.rtol = reinterpret_cast<const double*>(x + s->X.rtol);
  v.maxit = reinterpret_cast<const int64_t*>(x + s->X.maxit);
  v.cancel = s->d_cancel;
  v.n = max_points;
  v.nb = max_requests;
  s->bufs[0] = x + s->X.means;
  s->bufs[1] = w + P.means2;
  if (mixed) {
    s->mixed = true;
    s->ops32 = ops32;
    s->maxiters_f32 = maxiters_f32;
    s->rtol_f32 = rtol_f32;
    s->settle_f32 = settle_f32;
    s->sh32 = s->sh;
    s->sh32.esz = 4;
    s->sh32.team = ops32->tsn;
    s->sh32.team_up = ops32->tsw;
    s->M = mixed_serve_layout(D, d, max_requests, max_points, s->level_cap);
    s->mw = x + align_up(s->X.total);
    s->h_done32.assign(max_requests, 1);
    const MixedServe& M = s->M;
    char* w32 = s->mw + M.p32;
    BatchRaw& b = s->a32;
    b.params = nullptr;  // the float64 parameters go to lin_mixed
    b.x0m = s->mw + M.x0m32;
    b.x0L = s->mw + M.x0L32;
    b.F = s->mw + M.F32;
    b.QL = s->mw + M.QL32;
    b.H = w32 + M.P32.H;
    b.c = w32 + M.P32.c;
    b.selem = w32 + M.P32.selem;
    b.chols = s->mw + M.chols32;
    b.pscal = reinterpret_cast<double*>(w32 + M.P32.pscal);
    b.pscale = reinterpret_cast<double*>(w32 + M.P32.pscale);
    b.frozen = reinterpret_cast<int32_t*>(w32 + M.P32.frozen);  // the float32 phase is over (done32)
    b.nactive = reinterpret_cast<int32_t*>(w32 + M.P32.nactive);
    b.maxiters = 0;
    b.rtol = 1e-6;
    b.atol = 1e-9;
    b.mrtol = 1e-13;
    b.matol = 1e-8;
    b.calibrate = false;
    b.team = s->sh32.team;
    b.lw = s->mw + M.lw32;
    BView& u = b.v;
    u = v;  // the float64 engine's per-request tables (offsets, fields, Nordsieck scales)
    u.frozen = b.frozen;
    u.rtol = nullptr;
    u.maxit = nullptr;
    const unsigned gq = (unsigned)((D * D + 255) / 256);
    ks_d2f<<<gq, 256, 0, s->st>>>(F, reinterpret_cast<float*>(s->mw + M.F32), (int64_t)D * D);
    ks_d2f<<<gq, 256, 0, s->st>>>(QL, reinterpret_cast<float*>(s->mw + M.QL32), (int64_t)D * D);
    int rc2 = cuda_status(cudaMemsetAsync(b.frozen, 0xff, sizeof(int32_t) * max_requests, s->st));
    if (!rc2) rc2 = launch_status();
    if (!rc2) rc2 = cuda_status(cudaStreamSynchronize(s->st));
    if (rc2) {
      pof_server_destroy(s);
      return rc2;
    }
  }
  *out = s;
  return POF_OK;
}

}  // namespace

extern "C" {

int pof_server_create(int32_t D, int32_t d, int64_t max_requests, int64_t max_points, size_t level_bytes,
                      const double* F, const double* QL, int32_t calibrate, void* workspace, size_t workspace_bytes,
                      pof_server** out) {
  return server_create(D, d, max_requests, max_points, level_bytes, F, QL, calibrate, false, 0, 1e-5, 1e300,
                       workspace, workspace_bytes, out);
}

int pof_server_create_mixed(int32_t D, int32_t d, int64_t max_requests, int64_t max_points, size_t level_bytes,
                            const double* F, const double* QL, int32_t calibrate, int64_t maxiters_f32,
                            double rtol_f32, double settle_f32, void* workspace, size_t workspace_bytes,
                            pof_server** out) {
  return server_create(D, d, max_requests, max_points, level_bytes, F, QL, calibrate, true, maxiters_f32, rtol_f32,
                       settle_f32, workspace, workspace_bytes, out);
}

int pof_server_destroy(pof_server* s) {
  if (!s) return POF_ERR_ARG;
  cudaStreamSynchronize(s->st);
  cudaStreamDestroy(s->st);
  if (s->h_cancel) cudaFreeHost(const_cast<int32_t*>(s->h_cancel));
  delete s;
  return POF_OK;
}

int64_t pof_server_submit(pof_server* s, int64_t n_steps, int32_t field, const double* params, double h,
                          const double* x0_mean, const double* x0_chol, const double* init_row, int64_t maxiters,
                          double rtol) {
  if (!s || !params || !x0_mean || !init_row || n_steps < 1 || maxiters < 0 || !(rtol >= 0) || !(h != 0.0))
    return POF_ERR_ARG;
  if (field <= 0 || field >= FIELD_COUNT || field_dim(field) != s->d) return POF_ERR_FIELD;
  double p01[2];
  if (!nordsieck_scales(s->D, s->d, h, &p01[0], &p01[1])) return POF_ERR_ARG;
  int64_t b = -1;
  for (int64_t i = 0; i < s->maxB; ++i)
    if (!s->slots[i].used) {
      b = i;
      break;
    }
  if (b < 0) return POF_ERR_BUSY;
  const int64_t g0 = s->arena.alloc(n_steps + 1);
  if (g0 < 0) return POF_ERR_BUSY;
  // the plan with this request must fit the level part
  s->h_gb[b] = g0;
  s->h_ns[b] = n_steps;
  s->h_c0[b] = serve_c0(n_steps);
  {
    std::vector<int32_t> act;
    for (int64_t i = 0; i < s->maxB; ++i)
      if ((s->slots[i].used && !s->slots[i].finished) || i == b) act.push_back((int32_t)i);
    BatchLevels Lt = batch_levels(s->sh, act, s->h_ns.data(), s->h_gb.data(), s->h_c0.data(), nullptr);
    if (Lt.total > s->level_cap || Lt.cnt[Lt.nlev] != Lt.Ba) {
      s->arena.release(g0, n_steps + 1);
      return POF_ERR_BUSY;
    }
  }
  const int D = s->D;
  AdmitBlock blk{};
  blk.gb = g0;
  blk.ns = n_steps;
  blk.maxit = maxiters;
  blk.fld = field;
  blk.p01[0] = p01[0];
  blk.p01[1] = p01[1];
  for (int k = 0; k < 4; ++k) blk.params[k] = params[k];
  blk.rtol = rtol;
  std::vector<double> rows(D + D + D * D, 0.0);
  memcpy(rows.data(), init_row, sizeof(double) * D);
  memcpy(rows.data() + D, x0_mean, sizeof(double) * D);
  if (x0_chol) memcpy(rows.data() + 2 * D, x0_chol, sizeof(double) * D * D);
  char* x = s->xw;
  const BatchPersist& P = s->P;
  char* w = s->w;
  int rc = cuda_status(cudaMemcpyAsync(x + s->X.admit, &blk, sizeof(blk), cudaMemcpyHostToDevice, s->st));
  if (!rc)
    rc = cuda_status(
        cudaMemcpyAsync(x + s->X.row, rows.data(), sizeof(double) * rows.size(), cudaMemcpyHostToDevice, s->st));
  if (rc) {
    s->arena.release(g0, n_steps + 1);
    return rc;
  }
  const int64_t N = n_steps + 1;
  const unsigned grid = (unsigned)((N * D + 255) / 256 < 1024 ? (N * D + 255) / 256 : 1024);
  ks_admit<<<grid, 256, 0, s->st>>>(
      (int32_t)b, reinterpret_cast<const AdmitBlock*>(x + s->X.admit), reinterpret_cast<const double*>(x + s->X.row),
      D, reinterpret_cast<int64_t*>(w + P.gb), reinterpret_cast<int64_t*>(w + P.ns),
      reinterpret_cast<int32_t*>(w + P.fld), reinterpret_cast<double*>(w + P.p01),
      reinterpret_cast<double*>(x + s->X.params), reinterpret_cast<double*>(x + s->X.rtol),
      reinterpret_cast<int64_t*>(x + s->X.maxit), reinterpret_cast<double*>(x + s->X.x0m),
      reinterpret_cast<double*>(x + s->X.x0L), reinterpret_cast<double*>(w + P.pscal),
      reinterpret_cast<double*>(w + P.pscale), reinterpret_cast<int32_t*>(w + P.frozen),
      static_cast<double*>(s->bufs[s->cur]));
  const bool phase32 = s->mixed && s->maxiters_f32 > 0;
  if (phase32) {
    const MixedServe& M = s->M;
    ks_admit_mixed<<<grid, 256, 0, s->st>>>(
        (int32_t)b, reinterpret_cast<const AdmitBlock*>(x + s->X.admit), reinterpret_cast<const double*>(x + s->X.row),
        D, s->mcur(), reinterpret_cast<double*>(s->mw + M.keep), reinterpret_cast<float*>(s->mw + M.x0m32),
        reinterpret_cast<float*>(s->mw + M.x0L32), s->mst(), s->a32.frozen, reinterpret_cast<int32_t*>(w + P.frozen));
  }
  rc = launch_status();
  // blk and rows are host memory of this frame, and the staging area is
  // reused by the next admission
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s->st));
  if (rc) {
    s->arena.release(g0, n_steps + 1);
    return rc;
  }
  Slot& sl = s->slots[b];
  s->h_cancel[b] = 0;  // no tick reads slot b's flag before the next re-plan
  sl.used = true;
  sl.finished = false;
  sl.g0 = g0;
  sl.ns = n_steps;
  sl.parity0 = s->cur;
  sl.phase32 = phase32;
  s->h_frozen[b] = phase32 ? 1 : 0;
  if (phase32) s->h_done32[b] = 0;
  s->dirty = true;
  return b;
}

int pof_server_launch(pof_server* s, int64_t iterations) {
  if (!s || iterations < 0) return POF_ERR_ARG;
  for (int64_t k = 0; k < iterations; ++k) {
    if (s->dirty) {
      int rc = s->replan();
      if (rc) return rc;
    }
    if (s->active.empty() && s->active32.empty()) return POF_OK;
    if (!s->active32.empty()) s->tick32();
    if (!s->active.empty()) {
      s->ops->iteration(s->a, s->bufs[s->cur], s->bufs[s->cur ^ 1], s->st);
      s->cur ^= 1;
    }
    ++s->ticks;
  }
  return launch_status();
}

int pof_server_sync(pof_server* s, int64_t* n_running) {
  if (!s) return POF_ERR_ARG;
  int rc = cuda_status(cudaMemcpyAsync(s->h_frozen.data(), s->a.frozen, sizeof(int32_t) * s->maxB,
                                       cudaMemcpyDeviceToHost, s->st));
  if (!rc && s->mixed)
    rc = cuda_status(cudaMemcpyAsync(s->h_done32.data(), s->a32.frozen, sizeof(int32_t) * s->maxB,
                                     cudaMemcpyDeviceToHost, s->st));
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s->st));
  if (rc) return rc;
  if (prof_on()) prof_flush();
  int64_t running = 0;
  for (int64_t b = 0; b < s->maxB; ++b) {
    Slot& sl = s->slots[b];
    if (!sl.used || sl.finished) continue;
    if (sl.phase32) {
      ++running;
      if (!s->h_done32[b]) continue;
      // float32 phase over: back to the input trajectory when float32 never
      // came within 100 rtol_f32 (pof_ieks_solve_batch_mixed's discard
      // rule), then the float64 iterations from the kept iterate
      const MixedServe& M = s->M;
      const int D = s->D;
      s->ops32->revert(1, s->a.v.gb + b, s->a.v.ns + b, s->mst() + (int64_t)M_COUNT * b, s->rtol_f32,
                       reinterpret_cast<const double*>(s->mw + M.keep), s->mcur(), s->st);
      rc = cuda_status(cudaMemcpyAsync(static_cast<double*>(s->bufs[s->cur]) + sl.g0 * D, s->mcur() + sl.g0 * D,
                                       sizeof(double) * D * (sl.ns + 1), cudaMemcpyDeviceToDevice, s->st));
      if (!rc) rc = cuda_status(cudaMemsetAsync(s->a.frozen + b, 0, sizeof(int32_t), s->st));
      if (!rc) rc = launch_status();
      if (rc) return rc;
      sl.phase32 = false;
      sl.parity0 = s->cur;
      s->h_frozen[b] = 0;
      s->dirty = true;
      continue;
    }
    if (s->h_frozen[b]) {
      sl.finished = true;
      s->done.push_back(b);
      s->dirty = true;
    } else {
      ++running;
    }
  }
  if (n_running) *n_running = running;
  return POF_OK;
}

int pof_server_step(pof_server* s, int64_t iterations, int64_t* n_running) {
  int rc = pof_server_launch(s, iterations);
  if (!rc) rc = pof_server_sync(s, n_running);
  return rc;
}

int pof_server_cancel(pof_server* s, int64_t slot) {
  if (!s || slot < 0 || slot >= s->maxB) return POF_ERR_ARG;
  const Slot& sl = s->slots[slot];
  if (!sl.used || sl.finished) return POF_ERR_ARG;
  s->h_cancel[slot] = 1;
  return POF_OK;
}

int64_t pof_server_poll(pof_server* s, int64_t* slots_out, int64_t cap) {
  if (!s || (cap > 0 && !slots_out)) return POF_ERR_ARG;
  const int64_t n = (int64_t)s->done.size() < cap ? (int64_t)s->done.size() : cap;
  for (int64_t i = 0; i < n; ++i) slots_out[i] = s->done[i];
  s->done.erase(s->done.begin(), s->done.begin() + n);
  return n;
}

int pof_server_fetch(pof_server* s, int64_t slot, double* means, double* chols, double* info) {
  if (!s || slot < 0 || slot >= s->maxB || !means || !chols) return POF_ERR_ARG;
  Slot& sl = s->slots[slot];
  if (!sl.used || !sl.finished) return POF_ERR_ARG;
  const int64_t N = sl.ns + 1;
  const int D = s->D;
  const unsigned grid = (unsigned)((N * D * D + 255) / 256 < 1024 ? (N * D * D + 255) / 256 : 1024);
  ks_fetch<<<grid, 256, 0, s->st>>>((int32_t)slot, sl.parity0, s->a.v.gb, s->a.v.ns,
                                    static_cast<const double*>(s->bufs[0]), static_cast<const double*>(s->bufs[1]),
                                    static_cast<const double*>(s->a.chols), s->a.pscal, s->a.pscale,
                                    s->calibrate ? 1 : 0, D, means, chols, info);
  int rc = launch_status();
  if (!rc) rc = cuda_status(cudaStreamSynchronize(s->st));
  if (rc) return rc;
  s->arena.release(sl.g0, N);
  sl = Slot();
  s->h_frozen[slot] = 1;
  return POF_OK;
}

int pof_server_mixed_info(pof_server* s, int64_t slot, double* info_f32) {
  if (!s || !s->mixed || slot < 0 || slot >= s->maxB || !info_f32) return POF_ERR_ARG;
  const Slot& sl = s->slots[slot];
  if (!sl.used || !sl.finished) return POF_ERR_ARG;
  ks_mixed_info<<<1, 32, 0, s->st>>>(s->mst(), (int32_t)slot, info_f32);
  return launch_status();
}

void* pof_server_stream(pof_server* s) { return s ? static_cast<void*>(s->st) : nullptr; }

}  // extern "C"
