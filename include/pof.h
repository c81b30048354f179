/*
 * pof.h -- C ABI of the GB300 (sm_103a) parallel-in-time IEKS library
 * (libpof.so).
 *
 * The reference (nathanaelbosch/parallel-in-time-ode-filters, package `pof`)
 * is a JAX library with no FFI of its own; its hot path is a set of Python
 * functions over JAX arrays.  Each entry point below replaces one of those
 * functions and keeps its argument meaning; a JAX-FFI or ctypes binding
 * passes device pointers straight through.
 *
 * Conventions
 *  - All array arguments are DEVICE pointers, row-major, C-contiguous, of the
 *    element type selected by `dtype` (POF_F64: double, POF_F32: float),
 *    except `out_scalars` / `info`, which are always device double arrays.
 *  - n_steps = N - 1 time steps, D = d (q + 1) state dimension, d the ODE /
 *    observation dimension.  Shapes: x0_mean (D), x0_chol (D, D);
 *    F, QL (D, D) when ft_stride == 0, else (n_steps, D, D) with
 *    ft_stride == D*D; H (n_steps, d, D); c (n_steps, d);
 *    R (d, d) when r_stride == 0, (n_steps, d, d) when r_stride == d*d, or
 *    NULL for R = 0; means (N, D); chols (N, D, D).
 *  - `stream` is a cudaStream_t (NULL: the legacy default stream).  All work
 *    is enqueued on it; calls return without waiting unless stated.
 *  - The caller owns every buffer, including the workspace (size from the
 *    matching *_workspace_bytes query).  The library allocates no device
 *    memory.
 *  - Return value: POF_OK (0), a negative usage / CUDA error, never a trap.
 *    Numerical failure (NaN) propagates into the outputs, as in the
 *    reference, and is reported through the scalars.
 */
#ifndef POF_H_
#define POF_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  POF_OK = 0,
  POF_ERR_ARG = -1,       /* null pointer, non-positive size, bad stride */
  POF_ERR_SHAPE = -2,     /* (D, d) combination not compiled into this build */
  POF_ERR_WORKSPACE = -3, /* workspace smaller than *_workspace_bytes */
  POF_ERR_CUDA = -4,      /* a CUDA runtime call failed (see pof_last_cuda_error) */
  POF_ERR_FIELD = -5,     /* unknown built-in field or d mismatch */
  POF_ERR_DTYPE = -6,     /* dtype not POF_F64 / POF_F32 */
  POF_ERR_BUSY = -7       /* no free request slot or memory right now (pof_server_submit) */
};

enum { POF_F64 = 0, POF_F32 = 1 };

/* Layout of the `out_scalars` block written by the filter/smoother entry
 * points (device doubles). */
enum {
  POF_S_NLL = 0,      /* -sum log N(obs) of the filter (filter.py:96-102)   */
  POF_S_OBJ = 1,      /* smoother objective (smoother.py:20)                */
  POF_S_SSQ = 2,      /* sigma^2 (filter.py:105-114, whiten quirk)           */
  POF_S_FOBJ = 3,     /* filter objective (filter.py:43-45)                 */
  POF_S_NOTCLOSE = 4, /* # mean entries not isclose(old, new, 1e-13, 1e-8) */
  POF_S_COUNT = 8
};

/* Layout of the `info` block written by pof_ieks_solve, per problem by the
 * batched solves and by pof_server_fetch (device doubles). */
enum {
  POF_I_ITERATIONS = 0,
  POF_I_NLL = 1,
  POF_I_OBJ = 2,
  POF_I_SSQ = 3,
  POF_I_STATUS = 4, /* POF_SOLVE_*: why the IEKS loop of this problem stopped */
  POF_I_COUNT = 5
};

/* Per-problem outcome of an IEKS loop (info[POF_I_STATUS]).  The loop stops
 * as the reference's does (pof/solver.py:36-45 with crit,
 * pof/convergence_criteria.py:4-13: on NaN, on convergence, or after
 * maxiters + 1 iterations); the status says which.  NaN and infinities stay
 * in the outputs -- nothing traps.  No reference counterpart (the reference
 * returns only the iteration count). */
enum {
  POF_SOLVE_CONVERGED = 0, /* crit held with finite objective and NLL */
  POF_SOLVE_MAXITERS = 1,  /* stopped after maxiters + 1 iterations without crit */
  POF_SOLVE_NONFINITE = 2, /* objective or NLL NaN or infinite (poisoned input, 0 pivot) */
  POF_SOLVE_CANCELLED = 3  /* pof_server_cancel before it stopped */
};

/* Built-in vector fields for on-device EK1 linearization (pof/ivp.py). */
enum {
  POF_FIELD_USER = 0,
  POF_FIELD_LOGISTIC = 1,       /* (r)                pof/ivp.py:7-14   */
  POF_FIELD_LOTKAVOLTERRA = 2,  /* (a, b, c, d)       pof/ivp.py:17-31  */
  POF_FIELD_VANDERPOL = 3,      /* (mu)               pof/ivp.py:34-41  */
  POF_FIELD_FITZHUGHNAGUMO = 4, /* (a, b, 1/tau, I)   pof/ivp.py:44-60  */
  POF_FIELD_FHN_CLASSIC = 5,    /* (a, b, c)                            */
  POF_FIELD_ROBER = 6,          /* (k1, k2, k3)       pof/ivp.py:63-79  */
  POF_FIELD_RIGID_BODY = 7,     /* (p0, p1, p2)       pof/ivp.py:82-90  */
  POF_FIELD_SEIR = 8,           /* (p0..p3)           pof/ivp.py:93-108 */
  POF_FIELD_THREEBODY = 9,      /* (mu)               pof/ivp.py:111-126 */
  POF_FIELD_HENONHEILES = 10,   /* (p)                pof/ivp.py:137-152 */
  /* (a, b, c, kv, kw): method-of-lines FitzHugh-Nagumo on a periodic 1-D grid
   * of m = d / 2 cells, y = (v_0..v_{m-1}, w_0..w_{m-1}),
   *   v_k' = c (v_k - v_k^3 / 3 + w_k) + kv (v_{k-1} - 2 v_k + v_{k+1}),
   *   w_k' = -(v_k - a + b w_k) / c + kw (w_{k-1} - 2 w_k + w_{k+1});
   * any even d (pof_linearize; no reference counterpart) */
  POF_FIELD_FHN_RD = 11
};

/* Text of a POF_* status; the last CUDA runtime error seen by libpof (for
 * POF_ERR_CUDA); the library's interface version.  No reference
 * counterpart (the reference raises Python exceptions). */
const char* pof_status_string(int status);
const char* pof_last_cuda_error(void);
int pof_version(void);

/* 1 if the (D, d) pair is compiled into this build's small-D tables, else 0
 * (uncompiled pairs with D >= 32 run on the dense path, see
 * pof_dense_linear_filtsmooth). */
int pof_shape_supported(int32_t D, int32_t d);

/* Bytes of the workspace of pof_linear_filtsmooth, pof_linear_noiseless_filtering
 * and pof_smoothing (0 when n_steps < 1 or D < 1).  The reference needs none:
 * XLA allocates the scan's intermediates (pof/parallel_filtsmooth/filter.py:35). */
size_t pof_filtsmooth_workspace_bytes(int32_t dtype, int64_t n_steps, int32_t D, int32_t d);

/* pof.parallel_filtsmooth.linear_filtsmooth(x0, dtm, dom)
 *   (pof/parallel_filtsmooth/__init__.py:5-10): filter then smoother.
 * Writes the smoothed states into out_mean (N, D) / out_chol (N, D, D) and
 * out_scalars[POF_S_NLL, POF_S_OBJ (smoother), POF_S_SSQ, POF_S_FOBJ]. */
int pof_linear_filtsmooth(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, const void* x0_mean,
                          const void* x0_chol, const void* F, const void* QL, int64_t ft_stride, const void* H,
                          const void* c, const void* R, int64_t r_stride, void* out_mean, void* out_chol,
                          double* out_scalars, void* workspace, size_t workspace_bytes, void* stream);

/* pof.parallel_filtsmooth.linear_noiseless_filtering(x0, dtm, dom)
 *   (pof/parallel_filtsmooth/filter.py:18-47): filtered states and
 * out_scalars[POF_S_NLL, POF_S_SSQ, POF_S_FOBJ] (the filter's obj is
 * reported in POF_S_FOBJ and copied to POF_S_OBJ). */
int pof_linear_noiseless_filtering(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, const void* x0_mean,
                                   const void* x0_chol, const void* F, const void* QL, int64_t ft_stride,
                                   const void* H, const void* c, const void* R, int64_t r_stride, void* out_mean,
                                   void* out_chol, double* out_scalars, void* workspace, size_t workspace_bytes,
                                   void* stream);

/* pof.parallel_filtsmooth.smoothing(dtm, filter_trajectory)
 *   (pof/parallel_filtsmooth/smoother.py:8-22): smoothed states from the
 * filtered ones (filt_mean/filt_chol, (N, D) / (N, D, D)); the smoother
 * objective goes to out_scalars[POF_S_OBJ]. */
int pof_smoothing(int32_t dtype, int64_t n_steps, int32_t D, const void* F, const void* QL, int64_t ft_stride,
                  const void* filt_mean, const void* filt_chol, void* out_mean, void* out_chol, double* out_scalars,
                  void* workspace, size_t workspace_bytes, void* stream);

/* The dense path: the filter and smoother above for large state dimensions.
 * pof_linear_filtsmooth, pof_linear_noiseless_filtering, pof_smoothing and
 * pof_filtsmooth_workspace_bytes take it by themselves for every (D, d)
 * with D >= 32 that pof_shape_supported reports as not compiled; these
 * entry points reach it for any shape and choose the number of chunks.
 * The reference's operators work at any D
 * (pof/parallel_filtsmooth/filter.py:117-142, smoother.py:53-63, tria
 * pof/utils.py:33-41); the small-D tables do not.  Same schedule as the
 * batched solve's (chunks fold their steps, the chunk totals are applied
 * one after the other from x0 / from the terminal state, every chunk then
 * runs the Kalman filter / RTS recursion from its start), each step a batch
 * of dense GEMMs, blocked Householder trias and triangular solves over the
 * chunks.  which: POF_DENSE_FILTER (pof_linear_noiseless_filtering),
 * POF_DENSE_FILTSMOOTH (pof_linear_filtsmooth), POF_DENSE_SMOOTHING
 * (pof_smoothing: x0_mean / x0_chol are the filtered means (N, D) / chols
 * (N, D, D); H, c, R unused).  chunks: the number of chunks (0: 64 in float64, 256 in
 * float32, or the POF_DENSE_CHUNKS environment variable; at most n_steps).  Arguments and
 * outputs otherwise as pof_linear_filtsmooth's. */
enum { POF_DENSE_FILTER = 0, POF_DENSE_FILTSMOOTH = 1, POF_DENSE_SMOOTHING = 2 };
size_t pof_dense_workspace_bytes(int32_t dtype, int32_t which, int64_t n_steps, int32_t D, int32_t d,
                                 int32_t chunks);
int pof_dense_linear_filtsmooth(int32_t which, int32_t dtype, int64_t n_steps, int32_t D, int32_t d,
                                const void* x0_mean, const void* x0_chol, const void* F, const void* QL,
                                int64_t ft_stride, const void* H, const void* c, const void* R, int64_t r_stride,
                                void* out_mean, void* out_chol, double* out_scalars, int32_t chunks, void* workspace,
                                size_t workspace_bytes, void* stream);

/* EK1 linearization of a built-in field at means[1:]
 *   (pof/step.py:12-22, pof/observations.py:35-40) with the Nordsieck-scaled
 * projections of pof/convenience.py:24-28 (step size h): writes
 * H (n_steps, d, D) and c (n_steps, d); cholR is zero.  `params` is a device
 * array of the field's parameters in `dtype`. */
int pof_linearize(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field, const void* params,
                  double h, const void* means, void* H, void* c, void* stream);

/* pof.sequential_filtsmooth.linear_filtsmooth(x0, dtm, dom)
 *   (pof/sequential_filtsmooth/__init__.py:13-16): the square-root Kalman
 * filter (filter.py:33-56) and RTS smoother (smoother.py:8-28) step after
 * step on one GPU thread -- the reference's sequential twin.  Writes the
 * smoothed states (the filtered ones when smooth == 0) and
 * out_scalars[POF_S_NLL] = +sum log-likelihood (the sequential twin's sign,
 * filter.py:23-30), [POF_S_OBJ] (0 when smooth == 0), [POF_S_SSQ].
 * No workspace. */
int pof_sequential_linear_filtsmooth(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, const void* x0_mean,
                                     const void* x0_chol, const void* F, const void* QL, int64_t ft_stride,
                                     const void* H, const void* c, const void* R, int64_t r_stride, int32_t smooth,
                                     void* out_mean, void* out_chol, double* out_scalars, void* stream);

/* pof.sequential_filtsmooth.filtsmooth(x0, dtm, om) for a built-in field
 *   (pof/sequential_filtsmooth/__init__.py:5-10): extended Kalman filter that
 * linearizes at each predicted mean (filter.py:9-30), then the RTS smoother.
 * Same outputs as pof_sequential_linear_filtsmooth; h is the step size of
 * the Nordsieck projections. */
int pof_sequential_eks(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field, const void* params,
                       double h, const void* x0_mean, const void* x0_chol, const void* F, const void* QL,
                       int64_t ft_stride, int32_t smooth, void* out_mean, void* out_chol, double* out_scalars,
                       void* stream);

/* Bytes of the workspace of pof_ieks_solve (0 when n_steps < 1 or D < 1). */
size_t pof_ieks_workspace_bytes(int32_t dtype, int64_t n_steps, int32_t D, int32_t d);

/* pof.solver.solve(f, y0, ts, order, init, calibrate, maxiters)
 *   (pof/solver.py:11-73) for a built-in field, in preconditioned
 * coordinates: the IEKS loop of solver.py:36-57 (ieks_step, step.py:33-45,
 * and crit, convergence_criteria.py:4-13) runs on the device.
 *   in:  means (N, D) the initial trajectory (pof/convenience.py:76-92), x0,
 *        F = QL-pair of the preconditioned IWP prior (constant, (D, D)).
 *   out: means (N, D), chols (N, D, D) -- the final states, calibrated twice
 *        when `calibrate` (solver.py:66-69); info[POF_I_*].
 * The loop runs as one CUDA graph with a while node (one iteration per pass
 * of its body, the loop condition set on the device), enqueued on `stream`
 * without waiting; the instantiated graph is kept for the next call with
 * the same arguments (per host thread).  With libpof's event profiler on,
 * POF_SOLVE_NO_GRAPH set, or maxiters above 100000 the iterations are
 * launched from the host instead, which waits on `stream` once per
 * iteration to read the loop condition. */
int pof_ieks_solve(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field, const void* params,
                   double h, const void* x0_mean, const void* x0_chol, const void* F, const void* QL, void* means,
                   void* chols, int64_t maxiters, int32_t calibrate, double* info, void* workspace,
                   size_t workspace_bytes, void* stream);

/* Bytes of the workspace of pof_ieks_solve_sequential (0 when n_steps < 1 or D < 1). */
size_t pof_ieks_sequential_workspace_bytes(int32_t dtype, int64_t n_steps, int32_t D, int32_t d);

/* pof.solver.solve(..., sequential=True) for a built-in field
 *   (pof/solver.py:11-73 with pof/step.py:37-40 dispatching to
 *   pof/sequential_filtsmooth/__init__.py:13-16): the IEKS loop of
 * pof_ieks_solve with the sequential square-root Kalman filter
 * (sequential_filtsmooth/filter.py:33-92) and RTS smoother (smoother.py:8-48)
 * in place of the parallel scans -- the same team kernels as the parallel
 * path's level 0, run over one chunk that spans the trajectory.  Arguments,
 * outputs and info as in pof_ieks_solve (nll with the parallel filter's
 * sign).  The loop is enqueued as pof_ieks_solve's is. */
int pof_ieks_solve_sequential(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, int32_t field,
                              const void* params, double h, const void* x0_mean, const void* x0_chol, const void* F,
                              const void* QL, void* means, void* chols, int64_t maxiters, int32_t calibrate,
                              double* info, void* workspace, size_t workspace_bytes, void* stream);

/* Bytes of the workspace of pof_ieks_solve_mixed (0 when n_steps < 1 or D < 1). */
size_t pof_ieks_mixed_workspace_bytes(int64_t n_steps, int32_t D, int32_t d);

/* pof.solver.solve with precision="mixed".  Float32 iterations first: each
 * linearizes in float64 at the current float64 trajectory, row-normalizes the
 * noiseless observation model (same constraint, smaller range), runs the
 * filter and smoother in float32 and converts the means back; it is kept if
 * finite.  The float32 phase ends when the largest change of the projected
 * trajectory y = E0 m falls below rtol_f32 relative to max |y|, when that
 * change failed to shrink three times in a row once the smallest change so
 * far is below settle_f32 (pass HUGE_VAL to count from the first iteration;
 * a smaller value lets the first iterations from a crude initial trajectory
 * be non-monotone -- more float32 iterations, fewer float64 ones, and on
 * problems with several IEKS fixed points possibly another one than the
 * float64 loop from the same start), after a non-finite float32 iterate
 * (discarded) or after maxiters_f32 iterations; a float32 phase whose
 * smallest change never came within 100 rtol_f32 is dropped (float32 is too
 * coarse for that problem) and the float64 loop starts from the input
 * trajectory.  Otherwise the float64 loop of
 * pof_ieks_solve runs from the last kept trajectory with the reference's
 * criterion, so the result is a float64 IEKS fixed point.  No reference
 * counterpart (the reference is float64 throughout).  All arrays float64 as
 * in pof_ieks_solve; info has POF_I_COUNT + 2 entries: [POF_I_COUNT] the
 * number of kept float32 iterations (POF_I_ITERATIONS counts the float64
 * ones), [POF_I_COUNT + 1] the smallest relative change the float32 phase
 * reached.  Waits on `stream` once per float32 iteration; the float64
 * loop is enqueued as pof_ieks_solve's is. */
int pof_ieks_solve_mixed(int64_t n_steps, int32_t D, int32_t d, int32_t field, const double* params, double h,
                         const double* x0_mean, const double* x0_chol, const double* F, const double* QL,
                         double* means, double* chols, int64_t maxiters_f32, double rtol_f32, double settle_f32,
                         int64_t maxiters,
                         int32_t calibrate, double* info, void* workspace, size_t workspace_bytes, void* stream);

/* Scratch size of pof_linear_filtsmooth_noalloc (16 MiB per GPU). */
#define POF_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)

/* pof_linear_filtsmooth without a workspace argument.  It has no
 * counterpart in the reference: it exists for callers that cannot allocate
 * device memory -- plugin hosts that hand a library only its input and
 * output buffers, programs whose device memory belongs to another allocator
 * (a framework's caching pool), real-time loops that must not call
 * cudaMalloc after start-up -- and can only pass inputs and outputs.
 * Arguments and results are those of pof_linear_filtsmooth.
 *  - Scratch is a fixed 16 MiB device array inside libpof, held by every GPU
 *    that loads the library until the process exits.  Problems whose
 *    pof_filtsmooth_workspace_bytes exceeds POF_NOALLOC_SCRATCH_BYTES are
 *    refused with POF_ERR_WORKSPACE before any GPU work.  The largest
 *    n_steps that fit, float64 (float32): D = 3: 34212 (100400); D = 4:
 *    20296 (40112); D = 5: 13408 (26618); D = 6: 5778 (11482); D = 8: 3344
 *    (6660); D = 9: 2664 (5316); D = 10: 2176 (4341); the dense path's
 *    shapes (D >= 32) only small cases.  Bad dtypes, shapes and sizes get
 *    pof_linear_filtsmooth's statuses first.
 *  - The first call on a device looks up the array's address on that device
 *    (the current device); make that first call before any stream capture.
 *    The address is kept until the process exits: resetting the device
 *    (cudaDeviceReset) after that first call is not supported.
 *  - Every call shares the array: calls whose work overlaps on the GPU
 *    (other streams, other host threads) race and must be serialized by the
 *    caller.  Nothing needs clearing between calls.
 *  - It allocates no device memory. */
int pof_linear_filtsmooth_noalloc(int32_t dtype, int64_t n_steps, int32_t D, int32_t d, const void* x0_mean,
                                  const void* x0_chol, const void* F, const void* QL, int64_t ft_stride,
                                  const void* H, const void* c, const void* R, int64_t r_stride, void* out_mean,
                                  void* out_chol, double* out_scalars, void* stream);

/* Runtime bounds checks (the substitute for a memory sanitizer).  A build
 * with -DPOF_CHECKS (pof._build.build(checks=True): libpof_checked.so)
 * tests the element, step and problem indices of the global accesses the
 * kernels derive from sizes and plan tables; a failing check skips its
 * access and records the source line (in csrc) of the first failure.
 * pof_checks_compiled: 1 in such a build, else 0.  pof_checks_read: that
 * line (0: no failure; always 0 in the normal build), cleared when `reset`.
 * Waits for the device.  No reference counterpart. */
int pof_checks_compiled(void);
int pof_checks_read(uint64_t* line_out, int32_t reset);

/* Per-kernel timing.  When enabled, every libpof launch is bracketed by CUDA
 * events on its stream; pof_profile_read waits for them and returns the
 * summed milliseconds and launch counts per kernel kind (POF_PK_*), in
 * arrays of nkinds entries; returns the number of kinds.  One host thread. */
enum {
  POF_PK_LINEARIZE = 0, POF_PK_FILT_L0_REDUCE, POF_PK_FILT_REDUCE, POF_PK_FILT_TOP, POF_PK_FILT_DOWN,
  POF_PK_FILT_L0_DOWN, POF_PK_FILT_FINALIZE, POF_PK_SMO_L0_REDUCE, POF_PK_SMO_REDUCE, POF_PK_SMO_TOP,
  POF_PK_SMO_DOWN, POF_PK_SMO_L0_DOWN, POF_PK_SMO_FINALIZE, POF_PK_CONTROL, POF_PK_SEQUENTIAL, POF_PK_COUNT
};
void pof_profile_enable(int32_t on);
/* FP64 FMA throughput probe (the roofline denominator of the float64
 * kernels): blocks x threads threads each run 8 independent chains of
 * `iters` fused multiply-adds (16 * iters flops per thread). `sink` is a
 * device array of `blocks` doubles that is (almost) never written. */
int pof_fp64_probe(int64_t iters, int32_t blocks, int32_t threads, double* sink, void* stream);
/* Diagnostics: the double reciprocal and reciprocal square root the kernels
 * use for reflector scalars and diagonal solves (Newton-Raphson from a
 * single-precision seed), applied to x (n device doubles; rsqrt_out = 0 for
 * x <= 0). */
int pof_recip_check(int64_t n, const double* x, double* rcp_out, double* rsqrt_out, void* stream);
int pof_profile_read(double* ms_out, int64_t* count_out, int32_t nkinds, int32_t reset);

/* ---------------------------------------------------------------------------
 * Batched solves: B independent IVPs of one state shape (D, d) -- each with
 * its own number of steps, step size h, built-in field and parameters --
 * through one pipeline of launches per IEKS iteration, replayed from a CUDA
 * graph.  No counterpart in the reference (it solves one IVP per call,
 * pof/solver.py:11-73); per problem, the result is that of pof_ieks_solve's
 * loop (same linearization, filter/smoother, calibration and criterion),
 * computed by a chunked scan segmented at problem boundaries.  A problem's
 * result depends only on its own inputs and on (C0, Cg): not on the other
 * problems of the batch.  Converged problems stop iterating (they are
 * dropped from the plan once they hold half of its steps).
 *
 * Host arrays: n_steps (B), fields (B, POF_FIELD_*), h (B).  Device arrays,
 * of the dtype: params (B, 4) (first field_nparams used), x0_mean (B, D),
 * x0_chol (B, D, D) (preconditioned coordinates, as in pof_ieks_solve),
 * F, QL (D, D) (preconditioned IWP, the same for every h), means (G, D) with
 * G = sum(n_steps) + B (problem b's N_b = n_steps[b] + 1 grid points follow
 * those of problem b - 1; in: initial trajectories, out: results),
 * chols (G, D, D) out; info (B, POF_I_COUNT) device doubles.  C0 (steps per
 * level-0 chunk) and Cg (group size above) may be 0 for the defaults.
 * Shapes compiled: (D, d) in {(3,1), (4,1), (5,1), (6,2), (8,2), (10,2)}.
 * Waits on its own stream once per two iterations; ordered after the work
 * already on `stream`, and work later put on `stream` waits for it. */
size_t pof_batch_workspace_bytes(int32_t dtype, int64_t B, const int64_t* n_steps, int32_t D, int32_t d,
                                 int32_t C0, int32_t Cg);
int pof_ieks_solve_batch(int32_t dtype, int64_t B, const int64_t* n_steps, int32_t D, int32_t d,
                         const int32_t* fields, const void* params, const double* h, const void* x0_mean,
                         const void* x0_chol, const void* F, const void* QL, void* means, void* chols,
                         int64_t maxiters, int32_t calibrate, int32_t C0, int32_t Cg, double* info, void* workspace,
                         size_t workspace_bytes, void* stream);

/* pof_ieks_solve_mixed for a batch (no reference counterpart): per problem,
 * float32 IEKS iterations (float64 linearization at the float64 iterate,
 * float32 filter/smoother, the change judged in float64) under
 * pof_ieks_solve_mixed's stopping and discard rules, then the float64 loop
 * of pof_ieks_solve_batch from the kept iterate.  Arrays as in
 * pof_ieks_solve_batch, all float64; info_f32 (B, 2) device doubles
 * receives, per problem, the number of kept float32 iterations and the
 * smallest relative change the float32 phase reached (may be NULL). */
size_t pof_batch_mixed_workspace_bytes(int64_t B, const int64_t* n_steps, int32_t D, int32_t d, int32_t C0,
                                       int32_t Cg);
int pof_ieks_solve_batch_mixed(int64_t B, const int64_t* n_steps, int32_t D, int32_t d, const int32_t* fields,
                               const double* params, const double* h, const double* x0_mean, const double* x0_chol,
                               const double* F, const double* QL, double* means, double* chols, int64_t maxiters_f32,
                               double rtol_f32, double settle_f32, int64_t maxiters, int32_t calibrate, int32_t C0,
                               int32_t Cg, double* info, double* info_f32, void* workspace, size_t workspace_bytes,
                               void* stream);

/* ---------------------------------------------------------------------------
 * Continuous-batching engine (no reference counterpart): IEKS solves of one
 * state shape (D, d) are admitted while others iterate.  Each tick runs one
 * IEKS iteration (pof_ieks_solve's loop body, per request: own field,
 * parameters, step, maxiters and objective rtol of crit) over every
 * admitted, unfinished request with the batched segmented scan; finished
 * requests leave the plan and their memory is reused.  A request's chunk
 * length depends on its own step count only, so its result is bit-identical
 * alone and in any mix.  The engine owns a CUDA stream (pof_server_stream);
 * its calls are for one host thread.
 *
 * Memory: the caller's workspace, sized by pof_server_workspace_bytes for
 * up to max_requests requests holding up to max_points grid points in total
 * and level_bytes of scan levels (the admission budget: a request that does
 * not fit is refused with POF_ERR_BUSY and can be submitted again later). */
typedef struct pof_server pof_server;
size_t pof_server_workspace_bytes(int32_t D, int32_t d, int64_t max_requests, int64_t max_points,
                                  size_t level_bytes);
/* F, QL: device (D, D) preconditioned IWP (the same for every step size). */
int pof_server_create(int32_t D, int32_t d, int64_t max_requests, int64_t max_points, size_t level_bytes,
                      const double* F, const double* QL, int32_t calibrate, void* workspace, size_t workspace_bytes,
                      pof_server** out);
int pof_server_destroy(pof_server* s);

/* The engine with float32 bulk iterations and float64 polish per request
 * (no reference counterpart): every admitted request first runs float32 IEKS
 * iterations -- float64 EK1 linearization at its float64 iterate, float32
 * filter/smoother, the change judged in float64 -- under the float32-phase
 * rules of pof_ieks_solve_batch_mixed (maxiters_f32, rtol_f32, settle_f32,
 * the same discard rule), then the float64 loop with its own maxiters and
 * rtol, as on pof_server_create's engine.  Both phases of all requests run
 * in the same ticks.  A request's result is that of
 * pof_ieks_solve_batch_mixed with C0 = its own chunk length, alone and in
 * any mix.  Workspace from pof_server_mixed_workspace_bytes. */
size_t pof_server_mixed_workspace_bytes(int32_t D, int32_t d, int64_t max_requests, int64_t max_points,
                                        size_t level_bytes);
int pof_server_create_mixed(int32_t D, int32_t d, int64_t max_requests, int64_t max_points, size_t level_bytes,
                            const double* F, const double* QL, int32_t calibrate, int64_t maxiters_f32,
                            double rtol_f32, double settle_f32, void* workspace, size_t workspace_bytes,
                            pof_server** out);
/* A finished request of a mixed engine (before pof_server_fetch): device
 * array info_f32 (2 doubles) <- the float32 iterations it kept and the
 * smallest relative change its float32 phase reached. */
int pof_server_mixed_info(pof_server* s, int64_t slot, double* info_f32);
/* Admit a request (host arrays): field, params (4), step h, x0 (D) and its
 * chol (D, D, NULL = 0) in preconditioned coordinates, the initial
 * trajectory's row (D, repeated over the N = n_steps + 1 grid points:
 * "constant" init), maxiters and the objective rtol of crit.  Returns the
 * request's slot (>= 0) or a negative status (POF_ERR_BUSY: retry later). */
int64_t pof_server_submit(pof_server* s, int64_t n_steps, int32_t field, const double* params, double h,
                          const double* x0_mean, const double* x0_chol, const double* init_row, int64_t maxiters,
                          double rtol);
/* Enqueue `iterations` ticks; pof_server_sync waits for them and moves the
 * requests that stopped to the finished list (n_running: still iterating). */
int pof_server_launch(pof_server* s, int64_t iterations);
int pof_server_sync(pof_server* s, int64_t* n_running);
int pof_server_step(pof_server* s, int64_t iterations, int64_t* n_running);
/* Host-set cancel flag of an admitted request: the engine reads it at each
 * of its ticks (mapped host memory, no CUDA call here), so a request stops
 * at the first tick that runs after this call -- also one enqueued earlier
 * by pof_server_launch -- and finishes with info[POF_I_STATUS] =
 * POF_SOLVE_CANCELLED and its last iterate.  Fetch it like any finished
 * request.  POF_ERR_ARG for a free or finished slot. */
int pof_server_cancel(pof_server* s, int64_t slot);
/* Up to cap slots that finished since the last poll. */
int64_t pof_server_poll(pof_server* s, int64_t* slots_out, int64_t cap);
/* Copy a finished request's result -- means (N, D), calibrated chols
 * (N, D, D), info (POF_I_COUNT) into device arrays -- and free its slot. */
int pof_server_fetch(pof_server* s, int64_t slot, double* means, double* chols, double* info);
void* pof_server_stream(pof_server* s);

#ifdef __cplusplus
}
#endif

#endif /* POF_H_ */
