"""Benchmark: plain float64 parallel-in-time IEKS, one IVP per launch.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload NAME]

A step is one complete solve -- pof.solver.solve(f, y0, ts, order,
init="constant") iterated to the reference's convergence criterion -- of the
named workload (default: FitzHugh-Nagumo, (a, b, c) = (0.2, 0.2, 3), q = 3,
D = 8, on a uniform grid).  Metric: IVP*steps/s = (N - 1) / solve time.

value        device-resident: inputs already in HBM, the whole IEKS loop in
             libpof (pof_ieks_solve), per-solve CUDA events, L2 flushed
             between solves.
e2e          the same solve through the public API with host (numpy) inputs,
             results copied back to host memory.
roofline     the dominant kernel's achieved FP64 rate (flop model
             pof/_flops.py / its launch time from libpof's event profiler)
             against the FP64 FMA throughput measured on this GPU by
             pof_fp64_probe.
cpu_baseline the NumPy float64 oracle (the reference's algorithm) on a
             bounded sample of the same workload.
--impl reference  the CPU restatement of the reference (oracle) alone, on the
             same workload and metric (the reference itself needs JAX, which
             is not installed on these machines).

Blocks of the default line (skipped with --no-extras): config0 (the
reference's N = 1000 configuration), batched (4096 FitzHugh-Nagumo IVPs and
512 Van der Pol IVPs, float64 and float32 + float64 polish), served (a
Poisson stream through pof.serve.Server, p50/p99), dense (the
reaction-diffusion system at (D, d) = (640, 128): one IEKS iteration's work on
the dense path, float32 and float64).  Other workloads: --workload
scan_sweep / v100_table / mixed_lv_vdp / serve_stream / fhn_batch4096 /
rd_d640.

Multi-GPU: each rank solves its own copy of the workload (replicas; the path
does not shard a single solve), value = sum over ranks.
"""

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "parallel-in-time-ode-filters_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (ivp constructor (pof.ivp / oracle.ivp name, kwargs), t1, q, N)
    "fhn_q3_N16384": ("fhn_classic", {}, 100.0, 3, 2**14),
    "fhn_q3_N65536": ("fhn_classic", {}, 100.0, 3, 2**16),
    "fhn_q3_N262144": ("fhn_classic", {}, 100.0, 3, 2**18),
    "fhn_q3_N1048576": ("fhn_classic", {}, 100.0, 3, 2**20),
    "logistic_q3_N65536": ("logistic", {"r": 3.0}, 10.0, 3, 2**16),
    "logistic_q3_N1048576": ("logistic", {"r": 3.0}, 10.0, 3, 2**20),
    "fhn_q3_N1000": ("fhn_classic", {}, 100.0, 3, 1000),
}
DEFAULT_WORKLOAD = "fhn_q3_N65536"
MAXITERS = 10_000  # the reference's default (pof/solver.py:12)

# DRAM bytes (read + write) per launch of a workload's dominant kernel
# (dram__bytes_read.sum + dram__bytes_write.sum from one ncu capture of
# k_filt_l0_down_team<double, 8, 2, 8> on this workload; not measured by the
# bench run itself)
NCU_TRAFFIC = {("fhn_q3_N65536", "filt_l0_down"): 66.193664e6 + 108.293888e6}


def workload_config(workload):
    """The `config` object of a plain workload's line: the same dict in the
    GPU arm and in the reference arm (measured quantities such as the
    iteration count are reported beside it, not in it)."""
    name, kw, t1, q, N = WORKLOADS[workload]
    from oracle import ivp as oivp

    ivp = getattr(oivp, name)(**kw)
    d = ivp.y0.shape[0]
    return {"workload": workload, "ivp": name, "params": [float(x) for x in ivp.params], "y0": ivp.y0.tolist(),
            "q": q, "D": d * (q + 1), "N": N, "t1": t1, "init": "constant", "maxiters": MAXITERS,
            "criterion": "pof/convergence_criteria.py (obj rtol 1e-6, atol 1e-9; means rtol 1e-13)",
            "l2": "flushed between solves (256 MiB write)"}


def jprint(obj):
    print(json.dumps(obj), flush=True)


def max_over_ranks(x, world, device):
    """Largest x over the ranks of a replica run (the slowest rank sets the
    job's time); x itself when there is one rank.  All ranks must call it."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world, device):
    """Sum of x over the ranks (x itself with one rank).  All ranks call it."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# CPU: the oracle (NumPy float64 restatement of the reference)
# ---------------------------------------------------------------------------


def _oracle_iteration_s(workload, M=None):
    """Seconds of one oracle IEKS iteration (ieks_step, the reference's
    associative-scan order) on the first M steps of the workload's grid, the
    whole grid when M is None (run in a worker process)."""
    from oracle import ivp as oivp, solver as osolver

    name, kw, t1, q, N = WORKLOADS[workload]
    ivp = getattr(oivp, name)(**kw)
    ts = np.linspace(ivp.t0, t1, N)
    if M is not None:
        ts = ts[: M + 1]
    st = osolver.set_up_solver(ivp, ts, q)
    states = osolver.get_initial_trajectory(st, "constant")
    t0 = time.perf_counter()
    osolver.ieks_step(st, states)
    return time.perf_counter() - t0


class CpuReference:
    """The reference's algorithm (the NumPy float64 oracle: its
    associative-scan bracketing, LAPACK QR) on every host core: `procs`
    worker processes (spawned, one BLAS thread each) each run one IEKS
    iteration over the WHOLE grid of the workload at the same time, i.e.
    procs independent solves progressing in parallel.  One round is one
    timed sample; a solve's time is extrapolated from it as
    (round time / procs) x the iteration count of the solve."""

    def __init__(self, workload, procs=None):
        import concurrent.futures as cf
        import multiprocessing as mp

        self.workload = workload
        self.procs = procs or os.cpu_count() or 1
        self._saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
        for k in self._saved:
            os.environ[k] = "1"  # one core per worker
        self.ex = cf.ProcessPoolExecutor(self.procs, mp_context=mp.get_context("spawn"))

    def warm(self):
        """Start the workers and import the oracle (a 64-step iteration each)."""
        list(self.ex.map(_oracle_iteration_s, [self.workload] * self.procs, [64] * self.procs))

    def round(self):
        """Wall seconds of one round: every worker one whole-grid iteration."""
        t0 = time.perf_counter()
        list(self.ex.map(_oracle_iteration_s, [self.workload] * self.procs))
        return time.perf_counter() - t0

    def close(self):
        self.ex.shutdown()
        for k, v in self._saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v

    def describe(self, iterations):
        N = WORKLOADS[self.workload][4]
        return ("one IEKS iteration (ieks_step) of the oracle over the whole grid (%d steps) in each of %d "
                "processes at once per sample; a solve's time is extrapolated as sample time / %d x %d iterations "
                "(the float64 GPU solve's iteration count)" % (N - 1, self.procs, self.procs, iterations))


def cpu_sample(workload, iterations, rounds=1):
    """cpu_baseline of the GPU arm: CpuReference, `rounds` timed rounds."""
    ref = CpuReference(workload)
    try:
        ref.warm()
        walls = [ref.round() for _ in range(rounds)]
    finally:
        ref.close()
    N = WORKLOADS[workload][4]
    wall = float(np.median(walls))
    solve_s = wall / ref.procs * iterations
    return {"value": (N - 1) / solve_s, "solve_s": solve_s, "round_s": wall, "cores": ref.procs,
            "sample": ref.describe(iterations)}


def run_reference(args, workload):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    iters = EXPECTED_ITERATIONS.get(workload)
    if iters is None:
        jprint({"impl": "reference", "unavailable": "no measured IEKS iteration count for workload %s to "
                "extrapolate the CPU sample with" % workload})
        return
    name, kw, t1, q, N = WORKLOADS[workload]
    ref = CpuReference(workload)
    try:
        for _ in range(max(args.warmup, 1)):  # worker start-up and imports (64-step iterations)
            ref.warm()
        walls = [ref.round() for _ in range(args.steps)]
    finally:
        ref.close()
    wall = float(np.mean(walls))
    solve_s = wall / ref.procs * iters
    value = (N - 1) / solve_s
    jprint(
        {
            "impl": "reference",
            "metric": "IVP*steps/s (parallel IEKS solve, float64)",
            "value": value,
            "unit": "IVP*steps/s",
            "n_gpus": args.gpus,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": wall * 1e3,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic",
            "config": workload_config(workload),
            "step": "one sample: %d whole-grid IEKS iterations at once (one per core); ms_per_step is its wall "
                    "time" % ref.procs,
            "extrapolation": {"iterations_per_solve": iters, "solves_in_parallel": ref.procs,
                              "solve_s": solve_s},
            "cpu_baseline": {"value": value, "unit": "IVP*steps/s", "cores": ref.procs, "kind": "port",
                             "sample": ref.describe(iters)},
            "e2e": {"value": value, "unit": "IVP*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is JAX (not installed here); this arm times the NumPy float64 restatement of its "
                    "algorithm (oracle/) on every host core",
        }
    )


# IEKS iteration counts of the workloads as the float64 GPU solve measures
# them on a GB300 (the GPU arm reports its own count beside them); the CPU
# arm, which cannot finish these solves in minutes, extrapolates its
# per-step-iteration sample with them, so both arms price the same number of
# iterations.  FHN's count at large N moves with rounding (the problem is
# ill-conditioned there), so it is a measured figure, not a constant of the
# algorithm.
EXPECTED_ITERATIONS = {
    "fhn_q3_N16384": 141,
    "fhn_q3_N65536": 150,
    "logistic_q3_N65536": 38,
    "logistic_q3_N1048576": 40,
    "fhn_q3_N1000": 657,  # the oracle's own count (tree order) on this workload
}


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def fp64_peak(torch, lib, _lib):
    """FP64 FMA throughput of this GPU (GFLOP/s), pof_fp64_probe."""
    dev = torch.cuda.current_device()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, threads, iters = sms * 8, 256, 4096
    sink = torch.zeros(blocks, dtype=torch.float64, device="cuda")
    s = _lib.stream_handle()
    best = 0.0
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(lib.pof_fp64_probe(iters, blocks, threads, _lib.ptr(sink), s), "pof_fp64_probe")
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, 16.0 * iters * blocks * threads / (ms * 1e-3) / 1e9)
    return best


def run_gpu(args, workload):
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from pof import _build, _flops, _lib, ivp as pivp, solver as psolver
    from pof.convenience import get_initial_trajectory, set_up_solver

    _build.build(verbose=False)
    lib = _lib.lib()
    name, kw, t1, q, N = WORKLOADS[workload]
    p = getattr(pivp, name)(**kw)
    ts_host = np.linspace(p.t0, t1, N)
    setup = set_up_solver(f=p.f, y0=p.y0, ts=ts_host, order=q)
    init = get_initial_trajectory(setup, "constant")
    D = init.mean.shape[1]
    d = setup["iwp"].wiener_process_dimension
    n = N - 1
    fname, params = setup["om"].field
    dev = torch.device("cuda", local)
    means0 = init.mean.contiguous()
    means = torch.empty_like(means0)
    chols = torch.empty((N, D, D), dtype=torch.float64, device=dev)
    info = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
    prm = torch.tensor(params, dtype=torch.float64, device=dev)
    F = setup["dtm"].F[0].contiguous()
    QL = setup["dtm"].QL[0].contiguous()
    m0 = setup["x0"].mean.contiguous()
    L0 = setup["x0"].chol.contiguous()
    wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
    ws = _lib.workspace(wsb, dev)
    flush = torch.empty(256 * 2**20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    def solve_resident():
        means.copy_(means0)
        rc = lib.pof_ieks_solve(_lib.POF_F64, n, D, d, _lib.FIELDS[fname], _lib.ptr(prm), float(setup["dt"]),
                                _lib.ptr(m0), _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL), _lib.ptr(means),
                                _lib.ptr(chols), MAXITERS, 1, _lib.ptr(info), _lib.ptr(ws), wsb,
                                _lib.stream_handle())
        _lib.check(rc, "pof_ieks_solve")

    for _ in range(args.warmup):
        solve_resident()
    torch.cuda.synchronize()
    iterations = int(info[_lib.I_ITERATIONS].item())
    if args.solves_only:  # the launches of W + K solves and nothing else (ncu captures)
        for _ in range(args.steps):
            solve_resident()
        torch.cuda.synchronize()
        return

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # timed region: K solves, per-solve events, L2 flushed between solves
    times = []
    barrier()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            solve_resident()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        barrier()
    ms = max_over_ranks(float(np.mean(times)), world, dev)
    value = world * n / (ms * 1e-3)

    # mixed precision (float32 iterations + float64 polish) on the same
    # workload, timed the same way; error against the float64 result
    mixed = None
    if not args.no_mixed:
        ref_means = means.clone()
        mws_b = lib.pof_ieks_mixed_workspace_bytes(n, D, d)
        mws = _lib.workspace(mws_b, dev)
        minfo = torch.zeros(_lib.I_COUNT + 2, dtype=torch.float64, device=dev)

        def solve_mixed():
            means.copy_(means0)
            rc = lib.pof_ieks_solve_mixed(n, D, d, _lib.FIELDS[fname], _lib.ptr(prm), float(setup["dt"]),
                                          _lib.ptr(m0), _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL), _lib.ptr(means),
                                          _lib.ptr(chols), MAXITERS, 1e-5, args.f32_settle, MAXITERS, 1, _lib.ptr(minfo),
                                          _lib.ptr(mws), mws_b, _lib.stream_handle())
            _lib.check(rc, "pof_ieks_solve_mixed")

        for _ in range(args.warmup):
            solve_mixed()
        mtimes = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            solve_mixed()
            e1.record()
            e1.synchronize()
            mtimes.append(e0.elapsed_time(e1))
        mms = float(np.mean(mtimes))
        E0 = setup["E0"]
        ya, yb = means @ E0.T, ref_means @ E0.T
        err = float(((ya - yb).abs().max() / yb.abs().max()).item())
        mixed = {"value": world * n / (mms * 1e-3), "unit": "IVP*steps/s", "ms_per_step": mms,
                 "iterations_float32": int(minfo[_lib.I_COUNT].item()),
                 "best_change_float32": float(minfo[_lib.I_COUNT + 1].item()),
                 "iterations_float64": int(minfo[_lib.I_ITERATIONS].item()),
                 "max_rel_err_vs_float64": err, "speedup_vs_float64": ms / mms}
        del mws

    # per-kernel times of one more solve (profiler on; not part of the timing)
    _lib.profile_enable(True)
    _lib.profile_read(reset=True)
    solve_resident()
    torch.cuda.synchronize()
    prof = _lib.profile_read(reset=True)
    _lib.profile_enable(False)
    launches_per_solve = sum(c for _, c in prof.values()) + 3  # + init, final scale, info copy
    it_flops = _flops.iteration_flops(n, D, d)
    kern = {k: v for k, v in prof.items() if v[1] > 0 and k in it_flops}
    dom_kind = max(kern, key=lambda k: kern[k][0])
    dom_ms_per_launch = kern[dom_kind][0] / kern[dom_kind][1]
    C0, cnt = _flops.plan_levels(n, D)
    launches_per_iter_dom = kern[dom_kind][1] / iterations
    dom_flops = it_flops[dom_kind] / launches_per_iter_dom
    peak = fp64_peak(torch, lib, _lib)
    achieved = dom_flops / (dom_ms_per_launch * 1e-3) / 1e9
    total_prof_ms = sum(v[0] for v in prof.values())

    # end to end through the public API with host inputs / outputs
    e2e_times = []
    h2d = d2h = 0
    y0_host = p.y0.numpy()
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ys, inf = psolver.solve(f=p.f, y0=y0_host, ts=ts_host, order=q, init="constant", maxiters=MAXITERS)
        m_host = ys.mean.cpu().numpy()
        c_host = ys.chol.cpu().numpy()
        it_host = int(inf["iterations"])
        el = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(el)
        h2d = ts_host.nbytes + y0_host.nbytes
        d2h = m_host.nbytes + c_host.nbytes + 8
    e2e_s = max_over_ranks(float(np.mean(e2e_times)), world, dev)
    e2e_value = world * n / e2e_s

    extras = {}
    if not args.no_extras:  # every rank: the batched block splits one batch over the ranks
        extras["config0"] = config0_block(args)
        extras["batched"] = batched_block(args)
        extras["served"] = served_block(args)
        if world == 1:
            try:  # a failure here must not cost the line its other numbers
                extras["dense"] = dense_block(args)
            except Exception as e:  # noqa: BLE001
                extras["dense"] = {"error": "%s: %s" % (type(e).__name__, e)}

    if rank != 0:
        return
    out = {
        "metric": "IVP*steps/s (parallel IEKS solve, float64)",
        "value": value,
        "unit": "IVP*steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(workload),
        "iterations": iterations,
        "status": _lib.solve_status(info[_lib.I_STATUS].item()),
        "ms_per_iteration": ms / iterations,
        "plan": {"C0": C0, "levels": cnt[1:]},
        "e2e": {"value": e2e_value, "unit": "IVP*steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                "path": "pof.solver.solve(numpy y0, ts) -> means/chols .cpu()"},
        "roofline": {"bound": "fp64", "kernel": dom_kind, "achieved": achieved, "peak": peak, "unit": "GFLOP/s",
                     "frac": achieved / peak, "traffic": NCU_TRAFFIC.get((workload, dom_kind)),
                     "traffic_source": ("ncu capture of this kernel on this workload (dram__bytes_read.sum + "
                                        "dram__bytes_write.sum per launch), a constant of bench.py, not measured "
                                        "in this run") if (workload, dom_kind) in NCU_TRAFFIC else None,
                     "algorithmic_bytes_per_launch": _flops.kernel_bytes(n, D, d).get(dom_kind),
                     "peak_source": "measured in this run by pof_fp64_probe (8 independent FP64 FMA chains per "
                                    "thread, all SMs); MEASURED_PEAKS.json has no FP64 figure",
                     "flops_per_launch": dom_flops, "ms_per_launch": dom_ms_per_launch},
        "kernels": {k: {"ms": round(v[0], 4), "launches": v[1]} for k, v in prof.items() if v[1]},
        "gpu_launches": int(launches_per_solve * args.steps),
        "solve_flops": sum(it_flops.values()) * iterations,
        "solve_gflops": sum(it_flops.values()) * iterations / (total_prof_ms * 1e-3) / 1e9,
        "reference_equivalent_gflops": _flops.reference_step_flops(D, d) * n * iterations / (ms * 1e-3) / 1e9,
        "clocks": clk.summary(),
    }
    if mixed is not None:
        out["mixed_precision"] = mixed
    out.update(extras)
    if not args.no_cpu_baseline:
        cb = cpu_sample(workload, iterations=iterations)
        out["cpu_baseline"] = {"value": cb["value"], "unit": "IVP*steps/s", "cores": cb["cores"], "kind": "port",
                               "sample": cb["sample"], "round_s": cb["round_s"]}
    jprint(out)


# ---------------------------------------------------------------------------
# Blocks of the default line: the other configurations, measured briefly
# ---------------------------------------------------------------------------

BATCH_BUDGET = 24  # maxiters of the default line's batched block: at most 25 IEKS iterations per instance


def _events_ms(torch, fn, reps):
    out = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    return out


def config0_block(args):
    """FitzHugh-Nagumo (0.2, 0.2, 3), t in [0, 100], N = 1000, q = 3,
    constant init, the reference's criterion: whole solves through
    pof_ieks_solve (inputs resident), 1 warm-up + 3 timed."""
    import torch

    from pof import _lib, ivp as pivp
    from pof.convenience import get_initial_trajectory, set_up_solver

    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    p = pivp.fhn_classic()
    N, q = 1000, 3
    ts = np.linspace(0.0, 100.0, N)
    setup = set_up_solver(f=p.f, y0=p.y0, ts=ts, order=q)
    means0 = get_initial_trajectory(setup, "constant").mean.contiguous()
    D, d, n = means0.shape[1], 2, N - 1
    means = torch.empty_like(means0)
    chols = torch.empty((N, D, D), dtype=torch.float64, device=dev)
    info = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
    prm = torch.tensor(setup["om"].field[1], dtype=torch.float64, device=dev)
    wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
    ws = _lib.workspace(wsb, dev)
    F, QL = setup["dtm"].F[0].contiguous(), setup["dtm"].QL[0].contiguous()
    m0, L0 = setup["x0"].mean.contiguous(), setup["x0"].chol.contiguous()

    def one():
        means.copy_(means0)
        _lib.check(lib.pof_ieks_solve(_lib.POF_F64, n, D, d, _lib.FIELDS["fhn_classic"], _lib.ptr(prm),
                                      float(setup["dt"]), _lib.ptr(m0), _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL),
                                      _lib.ptr(means), _lib.ptr(chols), MAXITERS, 1, _lib.ptr(info), _lib.ptr(ws), wsb,
                                      _lib.stream_handle()), "pof_ieks_solve")

    one()
    ms = float(np.mean(_events_ms(torch, one, 3)))
    it = int(info[_lib.I_ITERATIONS].item())
    return {"workload": "fhn_q3_N1000 (the reference's CPU configuration)", "ms_per_solve": ms, "iterations": it,
            "ms_per_iteration": ms / it, "value": n / (ms * 1e-3), "unit": "IVP*steps/s",
            "status": _lib.solve_status(info[_lib.I_STATUS].item()),
            "note": "the iteration count is decided by rounding on this problem (the reference's own tree and "
                    "sequential orders stop at 657 and another count); ms per iteration compares kernels"}


def batched_block(args):
    """The batched configuration's exact instances (4096 FitzHugh-Nagumo,
    default_rng(0), N log-uniform in [256, 8192], q = 3) under a fixed
    iteration budget (maxiters = BATCH_BUDGET): step-iterations/s of the
    plain one-solve-per-launch float64 path (8 instances stratified by N),
    the batched float64 solve and the batched mixed solve (float32 iterations
    under the same budget, float64 polish under it), each timed once after a
    one-iteration warm-up; per-instance error of mixed against batched
    float64."""
    import torch

    from pof import _lib, batch as pbatch

    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    rank, world, _ = dist_info()
    family, B, seed, q, _ = BATCH_WORKLOADS["fhn_batch4096"]
    problems = batch_problems(family, B, seed)
    if world > 1:  # one fixed batch split over the ranks by steps
        problems = [problems[b] for b in pbatch.shard([len(p[3]) - 1 for p in problems], world)[rank]]
    prep = pbatch.prepare_batch(problems, q, device=dev)
    Bl = prep["B"]
    n_steps = prep["n_steps"]
    D, d = prep["D"], prep["d"]
    means = torch.empty_like(prep["means0"])
    G = means.shape[0]
    chols = torch.empty((G, D, D), dtype=torch.float64, device=dev)
    info = torch.zeros((Bl, _lib.I_COUNT), dtype=torch.float64, device=dev)
    info32 = torch.zeros((Bl, 2), dtype=torch.float64, device=dev)
    ws = [None]

    def solve(precision, maxiters):
        means.copy_(prep["means0"])
        ws[0] = pbatch.run_batch(prep, means, chols, info, maxiters=maxiters, workspace=ws[0], precision=precision,
                                 info_f32=info32, maxiters_f32=maxiters, settle_f32=args.f32_settle)

    out = {"workload": "fhn_batch4096: %d instances%s, a, b, c within +-20%% of (0.2, 0.2, 3), y0 ~ N((-1, 1), "
                       "0.1^2 I), t in [0, 100], N log-uniform in [256, 8192] (default_rng(0)), q = 3"
                       % (B, " (this rank's share: %d)" % Bl if world > 1 else ""),
           "budget": "fixed iteration budget: maxiters = %d (at most %d IEKS iterations per instance; instances "
                     "that meet the criterion stop earlier)" % (BATCH_BUDGET, BATCH_BUDGET + 1),
           "total_steps": int(n_steps.sum())}
    def timed_all(fn):
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return max_over_ranks(_events_ms(torch, fn, 1)[0], world, dev)

    solve("float64", 0)
    t64 = timed_all(lambda: solve("float64", BATCH_BUDGET))
    its = info[:, _lib.I_ITERATIONS].cpu().numpy()
    st = info[:, _lib.I_STATUS].cpu().numpy()
    si64 = sum_over_ranks(float((n_steps * its).sum()), world, dev)
    steps_all = sum_over_ranks(float(n_steps.sum()), world, dev)
    ref = means.clone()
    out["batched_float64"] = {"ms": t64, "step_iterations_per_s": si64 / (t64 * 1e-3),
                              "ivp_steps_per_s": steps_all / (t64 * 1e-3),
                              "converged": int(sum_over_ranks(int((st == 0).sum()), world, dev))}
    solve("mixed", 0)
    tmx = timed_all(lambda: solve("mixed", BATCH_BUDGET))
    it64 = info[:, _lib.I_ITERATIONS].cpu().numpy()
    it32 = info32[:, 0].cpu().numpy()
    stm = info[:, _lib.I_STATUS].cpu().numpy()
    err = _project_err(prep, means, ref)
    both = (st == 0) & (stm == 0)
    out["batched_mixed"] = {
        "ms": tmx,
        "step_iterations_per_s": sum_over_ranks(float((n_steps * (it64 + it32)).sum()), world, dev) / (tmx * 1e-3),
        "ivp_steps_per_s": steps_all / (tmx * 1e-3),
        "iterations_float32_total": int(it32.sum()), "iterations_float64_total": int(it64.sum()),
        "converged": int((stm == 0).sum()),
        "rel_err_vs_batched_float64": {"max": float(err.max()), "median": float(np.median(err))},
        "rel_err_where_both_converged": {"instances": int(both.sum()),
                                         "max": float(err[both].max()) if both.any() else None,
                                         "median": float(np.median(err[both])) if both.any() else None,
                                         "fraction_within_1e-6": float((err[both] <= 1e-6).mean())
                                         if both.any() else None}}
    # plain float64 path, one pof_ieks_solve per instance, same budget
    order = np.argsort(n_steps)
    sample = [int(order[int(i)]) for i in np.linspace(0, Bl - 1, 8)]
    plain_ms, plain_si, plain_steps = 0.0, 0.0, 0
    for b in sample:
        n = int(n_steps[b])
        m = torch.empty((n + 1, D), dtype=torch.float64, device=dev)
        c = torch.empty((n + 1, D, D), dtype=torch.float64, device=dev)
        inf = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
        wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
        pws = _lib.workspace(wsb, dev)
        m0 = prep["means0"][prep["offsets"][b]:prep["offsets"][b + 1]]
        x0m, x0L = prep["x0m"][b].contiguous(), prep["x0L"][b].contiguous()

        def one():
            m.copy_(m0)
            _lib.check(lib.pof_ieks_solve(_lib.POF_F64, n, D, d, int(prep["fields"][b]), _lib.ptr(prep["params"][b]),
                                          float(prep["h"][b]), _lib.ptr(x0m), _lib.ptr(x0L), _lib.ptr(prep["F"]),
                                          _lib.ptr(prep["QL"]), _lib.ptr(m), _lib.ptr(c), BATCH_BUDGET, 1,
                                          _lib.ptr(inf), _lib.ptr(pws), wsb, _lib.stream_handle()), "pof_ieks_solve")

        one()
        t = _events_ms(torch, one, 1)[0]
        plain_ms += t
        plain_si += n * int(inf[_lib.I_ITERATIONS].item())
        plain_steps += n
    plain_rate = plain_si / (plain_ms * 1e-3)
    out["plain_float64"] = {"sample": "8 instances stratified by N, one pof_ieks_solve each",
                            "step_iterations_per_s": plain_rate, "ivp_steps_per_s": plain_steps / (plain_ms * 1e-3)}
    out["speedup_vs_plain"] = {
        "batched_float64": out["batched_float64"]["step_iterations_per_s"] / plain_rate,
        "batched_mixed": out["batched_mixed"]["step_iterations_per_s"] / plain_rate,
        "unit": "ratio of step-iterations/s under the same budget"}
    del ws[0]
    out["vanderpol_mixed"] = vdp_mixed_block(args)
    return out


def vdp_mixed_block(args):
    """The float32 + float64-polish form where float32 can carry the bulk of
    the iterations: 512 Van der Pol IVPs (mu within +-20 % of 1, y0 ~
    N((2, 0), 0.1^2 I), t in [0, 6.3], N log-uniform in [256, 8192], q = 3),
    solved to the reference's criterion (no budget): IVP*steps/s of the
    plain one-solve-per-launch float64 path (8 instances stratified by N),
    of the batched float64 and of the batched mixed solve, and the
    per-instance error of mixed against batched float64."""
    import torch

    from pof import _lib, batch as pbatch

    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    family, B, seed, q, maxiters = BATCH_WORKLOADS["vdp_batch512"]
    prep = pbatch.prepare_batch(batch_problems(family, B, seed), q, device=dev)
    n_steps = prep["n_steps"]
    D, d = prep["D"], prep["d"]
    means = torch.empty_like(prep["means0"])
    chols = torch.empty((means.shape[0], D, D), dtype=torch.float64, device=dev)
    info = torch.zeros((B, _lib.I_COUNT), dtype=torch.float64, device=dev)
    info32 = torch.zeros((B, 2), dtype=torch.float64, device=dev)
    ws = [None]

    def solve(precision):
        means.copy_(prep["means0"])
        ws[0] = pbatch.run_batch(prep, means, chols, info, maxiters=maxiters, workspace=ws[0], precision=precision,
                                 info_f32=info32, maxiters_f32=maxiters, settle_f32=args.f32_settle)

    solve("float64")
    t64 = float(np.median(_events_ms(torch, lambda: solve("float64"), 3)))
    ref = means.clone()
    it64 = info[:, _lib.I_ITERATIONS].cpu().numpy()
    ws[0] = None
    solve("mixed")
    tmx = float(np.median(_events_ms(torch, lambda: solve("mixed"), 3)))
    err = _project_err(prep, means, ref)
    it32 = info32[:, 0].cpu().numpy()
    order = np.argsort(n_steps)
    plain_ms, plain_steps = 0.0, 0
    for b in [int(order[int(i)]) for i in np.linspace(0, B - 1, 8)]:
        n = int(n_steps[b])
        m = torch.empty((n + 1, D), dtype=torch.float64, device=dev)
        c = torch.empty((n + 1, D, D), dtype=torch.float64, device=dev)
        inf = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
        wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
        pws = _lib.workspace(wsb, dev)
        m0 = prep["means0"][prep["offsets"][b]:prep["offsets"][b + 1]]
        x0m, x0L = prep["x0m"][b].contiguous(), prep["x0L"][b].contiguous()

        def one():
            m.copy_(m0)
            _lib.check(lib.pof_ieks_solve(_lib.POF_F64, n, D, d, int(prep["fields"][b]), _lib.ptr(prep["params"][b]),
                                          float(prep["h"][b]), _lib.ptr(x0m), _lib.ptr(x0L), _lib.ptr(prep["F"]),
                                          _lib.ptr(prep["QL"]), _lib.ptr(m), _lib.ptr(c), maxiters, 1,
                                          _lib.ptr(inf), _lib.ptr(pws), wsb, _lib.stream_handle()), "pof_ieks_solve")

        one()
        plain_ms += _events_ms(torch, one, 1)[0]
        plain_steps += n
    plain = plain_steps / (plain_ms * 1e-3)
    steps = float(n_steps.sum())
    return {"workload": "vdp_batch512: 512 Van der Pol IVPs, mu within +-20%% of 1, y0 ~ N((2, 0), 0.1^2 I), "
                        "t in [0, 6.3], N log-uniform in [256, 8192] (default_rng(0)), q = 3, the reference's "
                        "criterion (maxiters %d)" % maxiters,
            "plain_float64_ivp_steps_per_s": plain,
            "batched_float64": {"ms": t64, "ivp_steps_per_s": steps / (t64 * 1e-3),
                                "iterations_median": float(np.median(it64))},
            "batched_mixed": {"ms": tmx, "ivp_steps_per_s": steps / (tmx * 1e-3),
                              "float32_iterations_median": float(np.median(it32)),
                              "float64_iterations_median": float(np.median(info[:, _lib.I_ITERATIONS].cpu().numpy())),
                              "instances_with_float32_kept": int((it32 > 0).sum())},
            "speedup_vs_plain": {"batched_float64": steps / (t64 * 1e-3) / plain,
                                 "batched_mixed": steps / (tmx * 1e-3) / plain},
            "mixed_rel_err_vs_float64": {"max": float(err.max()), "median": float(np.median(err)),
                                         "fraction_within_1e-6": float((err <= 1e-6).mean())}}


def served_block(args):
    """A short served stream: 48 requests (logistic, FitzHugh-Nagumo,
    Lotka-Volterra, Van der Pol mu = 10; +-20 % parameters, N log-uniform in
    [2^8, 2^16], q in {2, 3, 4}, tolerance in {1e-4, 1e-6}, maxiters 100) at
    16 Poisson arrivals/s, served in real time by pof.serve.Server; latency
    percentiles and throughput against the plain path serving the same
    arrivals one request at a time (first come, first served, on each
    request's measured pof_ieks_solve time)."""
    import torch

    from pof import _lib, batch as pbatch, serve

    lib = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    R, rate, maxiters, seed = 48, 16.0, 100, 0
    reqs = serve_requests(R, seed)
    steps_total = sum(len(r[3]) - 1 for r in reqs)
    plain_t = []
    for (nm, p, y0, ts, q, tol) in reqs:
        prep = pbatch.prepare_batch([(nm, p, y0, ts)], q, device=dev)
        n, D, d = int(prep["n_steps"][0]), prep["D"], prep["d"]
        m = prep["means0"].clone()
        c = torch.empty((n + 1, D, D), dtype=torch.float64, device=dev)
        inf = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
        wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
        ws = _lib.workspace(wsb, dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _lib.check(lib.pof_ieks_solve(_lib.POF_F64, n, D, d, int(prep["fields"][0]), _lib.ptr(prep["params"][0]),
                                      float(prep["h"][0]), _lib.ptr(prep["x0m"][0]), _lib.ptr(prep["x0L"][0]),
                                      _lib.ptr(prep["F"]), _lib.ptr(prep["QL"]), _lib.ptr(m), _lib.ptr(c),
                                      maxiters, 1, _lib.ptr(inf), _lib.ptr(ws), wsb, _lib.stream_handle()),
                   "pof_ieks_solve")
        torch.cuda.synchronize()
        plain_t.append(time.perf_counter() - t0)
        del ws, m, c
    arrivals = np.cumsum(np.random.default_rng(seed + 1000).exponential(1.0 / rate, size=R))
    fin, lat_plain = 0.0, []
    for a, t in zip(arrivals, plain_t):
        fin = max(a, fin) + t
        lat_plain.append(fin - a)

    def stream(precision):
        srv = serve.Server(max_requests=256, max_points=1 << 21, device=dev, precision=precision,
                           settle_f32=args.f32_settle)
        for r in reqs[:6]:  # engines built and warmed
            nm, p, y0, ts, q, tol = r
            srv.submit(nm, p, y0, ts[: min(len(ts), 300)], q, rtol=tol, maxiters=maxiters)
        while srv.busy():
            srv.tick()
        srv.results.clear()
        t_start = time.perf_counter()
        rid_of, k = {}, 0
        while k < R or srv.busy():
            now = time.perf_counter() - t_start
            while k < R and arrivals[k] <= now:
                nm, p, y0, ts, q, tol = reqs[k]
                rid_of[srv.submit(nm, p, y0, ts, q, rtol=tol, maxiters=maxiters,
                                  t_arrival=t_start + arrivals[k])] = k
                k += 1
            if srv.busy():
                srv.tick()
            elif k < R:
                time.sleep(max(0.0, min(0.01, arrivals[k] - (time.perf_counter() - t_start))))
        lat = [srv.t_done[rid] - srv.t_submit[rid] for rid in rid_of]
        res = {rid_of[rid]: srv.result(rid) for rid in rid_of}
        makespan = max(srv.t_done[rid] for rid in rid_of) - (t_start + arrivals[0])
        srv.close()
        statuses = [res[i][1]["status"] for i in range(R)]
        return res, {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                     "ivp_steps_per_s": steps_total / makespan, "makespan_s": makespan,
                     "status_counts": {s_: statuses.count(s_) for s_ in sorted(set(statuses))}}

    res64, served64 = stream("float64")
    resmx, servedmx = stream("mixed")
    errs = []
    for i in range(R):
        (a, _), ia = resmx[i]
        (b, _), ib = res64[i]
        if ia["status"] == ib["status"] == "converged":
            errs.append(float((a - b).abs().max() / b.abs().max()))
    errs = np.array(errs) if errs else np.array([np.nan])
    servedmx["float32_iterations_total"] = int(sum(int(resmx[i][1]["iterations_float32"]) for i in range(R)))
    servedmx["rel_err_vs_served_float64"] = {"requests_both_converged": int(np.isfinite(errs).sum()),
                                             "max": float(np.nanmax(errs)), "median": float(np.nanmedian(errs)),
                                             "fraction_within_1e-6": float((errs <= 1e-6).mean())}
    servedmx["speedup_vs_plain_fifo"] = servedmx["ivp_steps_per_s"] / (steps_total / (fin - arrivals[0]))
    return {"workload": "%d requests at %.0f/s (Poisson), logistic / FitzHugh-Nagumo / Lotka-Volterra / Van der Pol "
                        "mu = 10, +-20 %% parameters, N log-uniform in [2^8, 2^16], q in {2, 3, 4}, tolerance in "
                        "{1e-4, 1e-6}, maxiters %d" % (R, rate, maxiters),
            "served": served64,
            "served_mixed": servedmx,
            "plain_fifo": {"p50_s": float(np.percentile(lat_plain, 50)), "p99_s": float(np.percentile(lat_plain, 99)),
                           "ivp_steps_per_s": steps_total / (fin - arrivals[0])},
            "omitted": "reaction-diffusion d = 128 requests: the serving engines batch the small-D kernels; the "
                       "dense path solves that system on its own (the default line's dense block, --workload "
                       "rd_d640 --dense-solve)"}


# ---------------------------------------------------------------------------
# Batched uneven solves: many FitzHugh-Nagumo IVPs in one batched solve
# ---------------------------------------------------------------------------

BATCH_WORKLOADS = {
    # name: (family, instances, seed, q, maxiters).  FHN: about one instance
    # in six cycles without meeting the reference's criterion (mostly N in
    # [512, 2048]) and runs to maxiters + 1, so the capped forms bound a
    # solve's length, and its IEKS has several fixed points per instance.
    # Van der Pol mu ~ 1: every instance converges, to one fixed point.
    "fhn_batch4096": ("fhn", 4096, 0, 3, MAXITERS),
    "fhn_batch4096_it100": ("fhn", 4096, 0, 3, 100),
    "fhn_batch512_it300": ("fhn", 512, 0, 3, 300),
    "vdp_batch512": ("vdp", 512, 0, 3, MAXITERS),
    "vdp_batch4096": ("vdp", 4096, 0, 3, MAXITERS),
}

BATCH_FAMILIES = {
    # family: (field, nominal params, y0 mean, t1, config description)
    "fhn": ("fhn_classic", (0.2, 0.2, 3.0), (-1.0, 1.0), 100.0,
            {"ivp": "fhn_classic", "params": "a, b, c uniform within +-20% of (0.2, 0.2, 3)",
             "y0": "N((-1, 1), 0.1^2 I)", "t1": 100.0}),
    "vdp": ("vanderpol", (1.0,), (2.0, 0.0), 6.3,
            {"ivp": "vanderpol", "params": "mu uniform within +-20% of 1", "y0": "N((2, 0), 0.1^2 I)", "t1": 6.3}),
}


def batch_problems(family, B, seed):
    """B IVPs of a family: each parameter uniform within +-20 % of its nominal
    value, y0 ~ N(y0 mean, 0.1^2 I), t in [0, t1], N log-uniform in
    [256, 8192] (seeded)."""
    field, p0, y0m, t1, _ = BATCH_FAMILIES[family]
    rng = np.random.default_rng(seed)
    prm = np.array(p0) * rng.uniform(0.8, 1.2, size=(B, len(p0)))
    y0 = np.array(y0m) + 0.1 * rng.standard_normal((B, len(y0m)))
    N = np.floor(np.exp(rng.uniform(np.log(256), np.log(8192), size=B))).astype(int)
    return [(field, tuple(prm[b]), y0[b], np.linspace(0.0, t1, N[b])) for b in range(B)]


def run_gpu_batch(args, workload):
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from pof import _build, _flops, _lib, batch as pbatch

    _build.build(verbose=False)
    lib = _lib.lib()
    family, B, seed, q, maxiters = BATCH_WORKLOADS[workload]
    problems = batch_problems(family, B, seed + rank)
    dev = torch.device("cuda", local)
    prep = pbatch.prepare_batch(problems, q, device=dev)
    n_steps = prep["n_steps"]
    total_steps = int(n_steps.sum())
    D, d = prep["D"], prep["d"]
    means0 = prep["means0"]
    G = means0.shape[0]
    means = torch.empty_like(means0)
    chols = torch.empty((G, D, D), dtype=torch.float64, device=dev)
    info = torch.zeros((B, _lib.I_COUNT), dtype=torch.float64, device=dev)
    ws = None

    def solve(precision="float64", info32=None):
        nonlocal ws
        means.copy_(means0)
        ws = pbatch.run_batch(prep, means, chols, info, maxiters=maxiters, workspace=ws, precision=precision,
                              info_f32=info32, maxiters_f32=maxiters, settle_f32=args.f32_settle)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps):
        out = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return out

    for _ in range(args.warmup):
        solve()
    if args.solves_only:  # the launches of W + K batched solves and nothing else (ncu captures)
        for _ in range(args.steps):
            solve()
        torch.cuda.synchronize()
        return
    barrier()
    with ClockSampler(local) as clk:
        times = timed(solve, args.steps)  # inputs (G x D means, ~0.5 GB) exceed L2
        barrier()
    ms = max_over_ranks(float(np.mean(times)), world, dev)
    its = info[:, _lib.I_ITERATIONS].cpu().numpy()
    step_iters = int((n_steps * its).sum())
    value = world * total_steps / (ms * 1e-3)
    ref_means = means.clone()

    # mixed precision: float32 iterations, float64 polish, per problem
    mixed = None
    if not args.no_mixed:
        info32 = torch.zeros((B, 2), dtype=torch.float64, device=dev)
        ws = None
        for _ in range(args.warmup):
            solve("mixed", info32)
        mt = timed(lambda: solve("mixed", info32), args.steps)
        mms = float(np.mean(mt))
        E0P = _project_err(prep, means, ref_means)
        it32 = info32[:, 0].cpu().numpy()
        it64 = info[:, _lib.I_ITERATIONS].cpu().numpy()
        # problems whose float64 solve met the criterion (not cut by maxiters)
        conv = its <= maxiters
        mixed = {"value": world * total_steps / (mms * 1e-3), "unit": "IVP*steps/s", "ms_per_step": mms,
                 "f32_settle": args.f32_settle,
                 "iterations_float32_total": int(it32.sum()), "iterations_float64_total": int(it64.sum()),
                 "problems_with_float32_kept": int((it32 > 0).sum()),
                 "rel_err_vs_float64": {"max": float(E0P.max()), "median": float(np.median(E0P)),
                                        "p90": float(np.percentile(E0P, 90)),
                                        "fraction_within_1e-6": float((E0P <= 1e-6).mean())},
                 "rel_err_vs_float64_where_float64_converged": {
                     "problems": int(conv.sum()),
                     "median": float(np.median(E0P[conv])) if conv.any() else None,
                     "fraction_within_1e-6": float((E0P[conv] <= 1e-6).mean()) if conv.any() else None,
                     "fraction_within_1e-4": float((E0P[conv] <= 1e-4).mean()) if conv.any() else None},
                 "speedup_vs_float64_batched": ms / mms}
        ws = None

    # plain one-solve-per-launch float64 path on a stratified sample
    order = np.argsort(n_steps)
    sample = [int(order[int(i)]) for i in np.linspace(0, B - 1, 8)]
    plain_s = 0.0
    plain_steps = 0
    for b in sample:
        n = int(n_steps[b])
        m = means0[prep["offsets"][b]:prep["offsets"][b + 1]].clone()
        c = torch.empty((n + 1, D, D), dtype=torch.float64, device=dev)
        inf = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
        wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
        pws = _lib.workspace(wsb, dev)
        x0m = prep["x0m"][b].contiguous()
        x0L = prep["x0L"][b].contiguous()

        def one():
            m.copy_(means0[prep["offsets"][b]:prep["offsets"][b + 1]])
            rc = lib.pof_ieks_solve(_lib.POF_F64, n, D, d, int(prep["fields"][b]), _lib.ptr(prep["params"][b]),
                                    float(prep["h"][b]), _lib.ptr(x0m), _lib.ptr(x0L), _lib.ptr(prep["F"]),
                                    _lib.ptr(prep["QL"]), _lib.ptr(m), _lib.ptr(c), maxiters, 1, _lib.ptr(inf),
                                    _lib.ptr(pws), wsb, _lib.stream_handle())
            _lib.check(rc, "pof_ieks_solve")

        one()
        tt = timed(one, 1)[0]
        plain_s += tt * 1e-3
        plain_steps += n
    plain_value = plain_steps / plain_s

    # per-kernel times of one batched solve (profiler on, not timed)
    _lib.profile_enable(True)
    _lib.profile_read(reset=True)
    solve()
    torch.cuda.synchronize()
    prof = _lib.profile_read(reset=True)
    _lib.profile_enable(False)
    per_step = {"filt_l0_down": _flops.kf_step(D, d, True) + _flops.objective_term(D),
                "filt_l0_reduce": _flops.cond_fold_step(D, d),
                "smo_l0_down": _flops.smooth_apply(D) + _flops.objective_term(D) + D * D}
    kern = {k: v for k, v in prof.items() if v[1] > 0 and k in per_step}
    dom = max(kern, key=lambda k: kern[k][0])
    dom_ms = kern[dom][0]
    dom_launches = kern[dom][1]
    achieved = per_step[dom] * step_iters / (dom_ms * 1e-3) / 1e9
    peak = fp64_peak(torch, lib, _lib)

    # end to end through the public API with host inputs and host results
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = pbatch.solve_batch(problems, order=q, maxiters=maxiters)
        ym = res.mean.cpu().numpy()
        yc = res.chol.cpu().numpy()
        el = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(el)
    h2d = sum(len(p[3]) * 8 + 16 + 24 for p in problems)
    d2h = ym.nbytes + yc.nbytes
    e2e_s = max_over_ranks(float(np.mean(e2e_times)), world, dev)

    if rank != 0:
        return
    out = {
        "metric": "IVP*steps/s (batched parallel IEKS solve, float64)",
        "value": value,
        "unit": "IVP*steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload, "instances": B, "seed": seed, **BATCH_FAMILIES[family][4],
                   "N": "log-uniform in [256, 8192]", "q": q, "D": D, "init": "constant",
                   "maxiters": maxiters, "total_steps": total_steps, "step_iterations": step_iters,
                   "iterations_percentiles": {str(p): float(np.percentile(its, p)) for p in (0, 50, 90, 99, 100)},
                   "l2": "inputs (%.2f GB of iterates) exceed L2" % (G * D * 8 / 1e9)},
        "plain_float64_one_solve_per_launch": {"value": plain_value, "unit": "IVP*steps/s",
                                               "sample": "8 instances stratified by N, pof_ieks_solve each",
                                               "speedup_batched_vs_plain": value / plain_value},
        "e2e": {"value": world * total_steps / e2e_s, "unit": "IVP*steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                "path": "pof.batch.solve_batch(problem list with numpy y0 / ts) -> means/chols .cpu()"},
        "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "peak_source": "measured on this GPU by pof_fp64_probe (FP64 FMA chains)",
                     "flops_total": per_step[dom] * step_iters, "ms_total": dom_ms, "launches": dom_launches},
        "kernels": {k: {"ms": round(v[0], 4), "launches": v[1]} for k, v in prof.items() if v[1]},
        "gpu_launches": int(sum(c for _, c in prof.values()) * args.steps),
        "clocks": clk.summary(),
    }
    if mixed is not None:
        out["mixed_precision"] = mixed
        out["plain_float64_one_solve_per_launch"]["speedup_mixed_batched_vs_plain"] = mixed["value"] / plain_value
    if not args.no_cpu_baseline:
        cb = cpu_sample_batch(problems, q, its)
        out["cpu_baseline"] = cb
    jprint(out)


def _project_err(prep, a, b):
    """Per problem, max |y_a - y_b| / max |y_b| over its solution components
    y = E0 P m (numpy array of B values)."""
    import torch

    counts = torch.as_tensor(prep["n_steps"] + 1, device=a.device)
    p0 = torch.repeat_interleave(prep["p0"].to(a.device), counts)[:, None]
    idx = torch.arange(prep["d"], device=a.device) * (prep["q"] + 1)
    ya, yb = a[:, idx] * p0, b[:, idx] * p0
    num = torch.segment_reduce((ya - yb).abs().amax(1), "max", lengths=counts)
    den = torch.segment_reduce(yb.abs().amax(1), "max", lengths=counts)
    return (num / den).cpu().numpy()


def cpu_sample_batch(problems, q, its, budget_s=20.0):
    """The oracle's cost per step and IEKS iteration on one instance of the
    batch (a contiguous sub-grid, as cpu_sample), extrapolated to every
    instance's steps x iterations."""
    from oracle import ivp as oivp, solver as osolver

    nm, p, y0, ts = problems[0]
    if nm == "fhn_classic":
        ivp = oivp.fhn_classic(tmax=float(ts[-1]), y0=list(y0), a=p[0], b=p[1], c=p[2])
    else:
        ivp = oivp.vanderpol(tmax=float(ts[-1]), y0=list(y0), stiffness_constant=p[0])
    M = 256
    while True:
        st = osolver.set_up_solver(ivp, ts[: M + 1], q)
        states = osolver.get_initial_trajectory(st, "constant")
        t0 = time.perf_counter()
        osolver.ieks_step(st, states)
        el = time.perf_counter() - t0
        if el > budget_s / 4 or M >= len(ts) - 1:
            break
        M = min(M * 4, len(ts) - 1)
    per = el / M
    total = sum((len(pp[3]) - 1) * int(i) for pp, i in zip(problems, its))
    steps = sum(len(pp[3]) - 1 for pp in problems)
    solve_s = per * total
    return {"value": steps / solve_s, "unit": "IVP*steps/s", "cores": 1, "kind": "port",
            "sample": "one IEKS iteration of the oracle on %d steps of instance 0; solve time extrapolated as cost "
                      "per step-iteration x sum over instances of steps x the GPU's iteration count" % M}


# ---------------------------------------------------------------------------
# Scan-length sweep: parallel IEKS solves against the sequential EKS pass on
# the same GPU, one IVP per launch
# ---------------------------------------------------------------------------

# The reference's published float64 IEKS results on a Tesla V100-SXM2-32GB
# (experiments/3_work_precision_diagram/data/<setup>_Tesla_V100-SXM2-32GB.csv:
# ms per solve, min of 3, and iterations), the rows the v100_table workload
# reruns: (ivp, q, N) -> (ms, iterations).
V100_PUBLISHED = {
    ("logistic", 3, 2**10): (55.8, 12), ("logistic", 3, 2**14): (143.4, 12), ("logistic", 3, 2**19): (2680.0, 12),
    ("fitzhughnagumo", 3, 2**10): (441.0, 62), ("fitzhughnagumo", 3, 2**14): (2523.0, 111),
    ("fitzhughnagumo", 3, 2**19): (54740.0, 112), ("vanderpol", 3, 2**19): (4829.0, 10),
    ("rigid_body", 3, 2**19): (11930.0, 10), ("henonheiles", 1, 2**19): (9494.0, 19),
}

SWEEP_WORKLOADS = {
    # name: (cases (field, kwargs, t1 or None for the IVP's own span, q, N values, largest N of the
    # sequential solves), unused, maxiters)
    "scan_sweep": ([("logistic", {"r": 3.0}, 10.0, q, [2**10, 2**12, 2**14, 2**16, 2**18, 2**20], 2**14)
                    for q in (1, 2, 3, 5)]
                   + [("fhn_classic", {}, 100.0, q, [2**10, 2**12, 2**14, 2**16], 2**10) for q in (1, 2, 3, 5)],
                   None, MAXITERS),
    # the rows of the reference's published V100 benchmark (pof.ivp default problems, constant init,
    # maxiters 1000) that fit the compiled shapes
    "v100_table": ([("logistic", {}, None, 3, [2**10, 2**14, 2**19], 0),
                    ("fitzhughnagumo", {}, None, 3, [2**10, 2**14, 2**19], 0),
                    ("vanderpol", {"stiffness_constant": 1.0}, None, 3, [2**19], 0),
                    ("rigid_body", {}, None, 3, [2**19], 0),
                    ("henonheiles", {"tmax": 10.0}, None, 1, [2**19], 0)], None, 1000),
}


def run_sweep(args, workload):
    """Wall time (device synchronized on both sides) per (IVP, q, N), one IVP
    per launch: the full parallel IEKS solve (pof.solver.solve, the
    reference's criterion), the full sequential IEKS solve on the same GPU
    (solve(sequential=True): the same loop with the square-root Kalman
    filter and RTS smoother run step after step by one team of the level-0
    kernels over a chunk spanning the grid) and one sequential extended
    Kalman smoother pass (pof.solver.sequential_eks_solve, one GPU thread
    running the EKF + RTS recursion; one linearization, not a solve)."""
    import torch

    from pof import _build, ivp as pivp, solver as psolver

    _build.build(verbose=False)
    cases, _, maxiters = SWEEP_WORKLOADS[workload]
    rows = []

    def wall(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, out

    for name, kw, t1, q, Ns, seq_max in cases:
        p = getattr(pivp, name)(**kw)
        for N in Ns:
            ts = np.linspace(p.t0, p.tmax, N) if t1 is None else np.linspace(0.0, t1, N)
            par = lambda: psolver.solve(f=p.f, y0=p.y0, ts=ts, order=q, init="constant", maxiters=maxiters)  # noqa: E731
            if N <= 2**16:
                wall(par)
            tp, (_, info) = wall(par)
            it = int(info["iterations"])
            row = {"ivp": name, "q": q, "D": int(p.y0.shape[0]) * (q + 1), "N": N, "parallel_ieks_ms": tp * 1e3,
                   "iterations": it, "parallel_ms_per_iteration": tp * 1e3 / max(it, 1),
                   "status": int(info["status"])}
            pub = V100_PUBLISHED.get((name, q, N)) if workload == "v100_table" else None
            if pub:
                row.update({"v100_published_ms": pub[0], "v100_published_iterations": pub[1],
                            "speedup_vs_v100_published": pub[0] / (tp * 1e3),
                            "per_iteration_speedup_vs_v100_published": (pub[0] / pub[1]) / (tp * 1e3 / max(it, 1))})
            if N <= seq_max:
                sq = lambda: psolver.solve(f=p.f, y0=p.y0, ts=ts, order=q, init="constant",  # noqa: E731
                                           maxiters=maxiters, sequential=True)
                tsi, (_, sinfo) = wall(sq)
                sit = int(sinfo["iterations"])
                row.update({"sequential_ieks_ms": tsi * 1e3, "sequential_iterations": sit,
                            "sequential_ms_per_iteration": tsi * 1e3 / max(sit, 1),
                            "parallel_speedup_per_iteration": (tsi / max(sit, 1)) / (tp / max(it, 1))})
                eks = lambda: psolver.sequential_eks_solve(f=p.f, y0=p.y0, ts=ts, order=q)  # noqa: E731
                wall(eks)
                te, _ = wall(eks)
                row["sequential_eks_pass_ms"] = te * 1e3
            rows.append(row)
            print(json.dumps(row), file=sys.stderr, flush=True)
    jprint({"metric": "ms per solve and per IEKS iteration, parallel vs sequential IEKS on the same GPU (float64, "
                      "one IVP per launch)",
            "value": None, "unit": "ms", "n_gpus": 1, "higher_is_better": False, "dtype": "f64",
            "data": "synthetic", "config": {"workload": workload, "init": "constant", "maxiters": maxiters,
                                            "timing": "wall clock, device synchronized, 1 warm-up for N <= 2^16"},
            "rows": rows})


# ---------------------------------------------------------------------------
# Served request stream: continuous batching against one-request-at-a-time
# ---------------------------------------------------------------------------

SERVE_WORKLOADS = {
    # name: (requests per rate, arrival rates (requests/s), seed, maxiters)
    "serve_stream": (96, (8.0, 32.0), 0, 300),
}

_SERVE_FIELDS = {
    # field: (parameters, y0, t1) before the +-20 % jitter of the parameters
    "logistic": ((3.0,), [0.01], 10.0),
    "fhn_classic": ((0.2, 0.2, 3.0), [-1.0, 1.0], 100.0),
    "lotkavolterra": ((1.5, 1.0, 3.0, 1.0), [1.0, 1.0], 10.0),
    "vanderpol": ((10.0,), [2.0, 0.0], 6.3),
}


def serve_requests(R, seed):
    """R requests: field uniform over logistic (d = 1), FitzHugh-Nagumo,
    Lotka-Volterra, Van der Pol mu = 10 (d = 2); parameters jittered
    uniformly within +-20 %; N log-uniform in [2^8, 2^16]; q in {2, 3, 4};
    objective tolerance in {1e-4, 1e-6}."""
    rng = np.random.default_rng(seed)
    names = sorted(_SERVE_FIELDS)
    out = []
    for _ in range(R):
        nm = names[rng.integers(len(names))]
        p, y0, t1 = _SERVE_FIELDS[nm]
        p = tuple(float(x) * rng.uniform(0.8, 1.2) for x in p)
        N = int(np.floor(np.exp(rng.uniform(np.log(2 ** 8), np.log(2 ** 16)))))
        q = int(rng.integers(2, 5))
        tol = 1e-4 if rng.uniform() < 0.5 else 1e-6
        out.append((nm, p, y0, np.linspace(0.0, t1, N), q, tol))
    return out


def run_serve(args, workload):
    """Poisson arrivals at each rate; the continuous-batching server in real
    time against the plain path (one pof_ieks_solve per request, first come
    first served, the same arrival times)."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from pof import _build, _lib, batch as pbatch, serve

    _build.build(verbose=False)
    lib = _lib.lib()
    R, rates, seed, maxiters = SERVE_WORKLOADS[workload]
    reqs = serve_requests(R, seed + rank)
    steps_total = sum(len(r[3]) - 1 for r in reqs)
    dev = torch.device("cuda", local)

    # plain path: each request's solve time, one at a time
    plain_t = []
    for (nm, p, y0, ts, q, tol) in reqs:
        prep = pbatch.prepare_batch([(nm, p, y0, ts)], q, device=dev)
        n, D, d = int(prep["n_steps"][0]), prep["D"], prep["d"]
        m = prep["means0"].clone()
        c = torch.empty((n + 1, D, D), dtype=torch.float64, device=dev)
        inf = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
        wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
        ws = _lib.workspace(wsb, dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.copy_(prep["means0"])
        _lib.check(lib.pof_ieks_solve(_lib.POF_F64, n, D, d, int(prep["fields"][0]), _lib.ptr(prep["params"][0]),
                                      float(prep["h"][0]), _lib.ptr(prep["x0m"][0]), _lib.ptr(prep["x0L"][0]),
                                      _lib.ptr(prep["F"]), _lib.ptr(prep["QL"]), _lib.ptr(m), _lib.ptr(c),
                                      maxiters, 1, _lib.ptr(inf), _lib.ptr(ws), wsb, _lib.stream_handle()),
                   "pof_ieks_solve")
        torch.cuda.synchronize()
        plain_t.append(time.perf_counter() - t0)
        del ws, m, c
    # warm the server's engines (first use builds them)
    srv = serve.Server(max_requests=256, max_points=1 << 21, device=dev)
    for r in reqs[:6]:
        nm, p, y0, ts, q, tol = r
        srv.submit(nm, p, y0, ts[: min(len(ts), 300)], q, rtol=tol, maxiters=maxiters)
    while srv.busy():
        srv.tick()

    lines = []
    rng = np.random.default_rng(seed + 1000)
    for rate in rates:
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=R))
        # plain: first come first served on the measured solve times
        fin = 0.0
        lat_plain = []
        for a, t in zip(arrivals, plain_t):
            start = max(a, fin)
            fin = start + t
            lat_plain.append(fin - a)
        makespan_plain = fin - arrivals[0]
        # served, in real time
        srv.results.clear()
        t_start = time.perf_counter()
        rid_of = {}
        k = 0
        while k < R or srv.busy():
            now = time.perf_counter() - t_start
            while k < R and arrivals[k] <= now:
                nm, p, y0, ts, q, tol = reqs[k]
                rid_of[srv.submit(nm, p, y0, ts, q, rtol=tol, maxiters=maxiters, t_arrival=t_start + arrivals[k])] = k
                k += 1
            if srv.busy():
                srv.tick()
            elif k < R:
                time.sleep(max(0.0, min(0.01, arrivals[k] - (time.perf_counter() - t_start))))
        lat = [srv.t_done[rid] - srv.t_submit[rid] for rid in rid_of]
        makespan = max(srv.t_done[rid] for rid in rid_of) - (t_start + arrivals[0])
        lines.append({
            "rate_per_s": rate,
            "served": {"p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
                       "throughput": steps_total / makespan, "makespan_s": makespan},
            "plain_fifo": {"p50_s": float(np.percentile(lat_plain, 50)), "p99_s": float(np.percentile(lat_plain, 99)),
                           "throughput": steps_total / makespan_plain, "makespan_s": makespan_plain},
        })
    srv.close()
    if rank != 0:
        return
    best = max(lines, key=lambda x: x["served"]["throughput"])
    jprint({
        "metric": "IVP*steps/s and p50/p99 latency, served request stream (continuous batching, float64)",
        "value": best["served"]["throughput"],
        "unit": "IVP*steps/s",
        "n_gpus": world,
        "steps": R,
        "warmup": 6,
        "ms_per_step": None,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload, "requests_per_rate": R, "seed": seed, "maxiters": maxiters,
                   "fields": "logistic, fhn_classic, lotkavolterra, vanderpol mu=10 (+-20 % parameters)",
                   "N": "log-uniform in [2^8, 2^16]", "q": [2, 3, 4], "tolerances": [1e-4, 1e-6],
                   "total_steps": steps_total,
                   "omitted": "reaction-diffusion d = 128 requests: the serving engines batch the small-D kernels; "
                              "the dense path solves that system on its own (--workload rd_d640 --dense-solve)"},
        "rates": lines,
        "plain_solve_s_total": float(sum(plain_t)),
    })


# ---------------------------------------------------------------------------
# Mixed precision with float64 polish on the problems of the mixed-precision
# configuration: Lotka-Volterra and Van der Pol mu in {1, 10, 100}, N = 2^14,
# q = 4 -- one solve per launch and batched, float64 and mixed
# ---------------------------------------------------------------------------

MIXED_WORKLOADS = {
    # name: ([(field, params, y0, t1)], N, q, maxiters).  Lotka-Volterra at
    # q = 4 on this grid does not converge in float64 (the iterates blow up
    # and the loop runs to maxiters), hence the cap.
    "mixed_lv_vdp": ([("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], 10.0),
                      ("vanderpol", (1.0,), [2.0, 0.0], 6.3),
                      ("vanderpol", (10.0,), [2.0, 0.0], 6.3),
                      ("vanderpol", (100.0,), [2.0, 0.0], 6.3)], 2 ** 14, 4, 1000),
}


def run_mixed(args, workload):
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from pof import _build, _lib, batch as pbatch

    _build.build(verbose=False)
    lib = _lib.lib()
    spec, N, q, maxiters = MIXED_WORKLOADS[workload]
    dev = torch.device("cuda", local)
    problems = [(nm, p, y0, np.linspace(0.0, t1, N)) for (nm, p, y0, t1) in spec]
    prep = pbatch.prepare_batch(problems, q, device=dev)
    B, D, d = prep["B"], prep["D"], prep["d"]
    off = prep["offsets"]
    steps = int(prep["n_steps"].sum())

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ts = []
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    results = {}
    # one solve per launch, float64 and mixed
    for prec in ("float64", "mixed"):
        per = []
        for b in range(B):
            n = int(prep["n_steps"][b])
            m = torch.empty((n + 1, D), dtype=torch.float64, device=dev)
            c = torch.empty((n + 1, D, D), dtype=torch.float64, device=dev)
            inf = torch.zeros(_lib.I_COUNT + 2, dtype=torch.float64, device=dev)
            if prec == "float64":
                wsb = lib.pof_ieks_workspace_bytes(_lib.POF_F64, n, D, d)
            else:
                wsb = lib.pof_ieks_mixed_workspace_bytes(n, D, d)
            ws = _lib.workspace(wsb, dev)
            m0 = prep["means0"][off[b]:off[b + 1]]
            args_c = (_lib.ptr(prep["params"][b]), float(prep["h"][b]), _lib.ptr(prep["x0m"][b]),
                      _lib.ptr(prep["x0L"][b]), _lib.ptr(prep["F"]), _lib.ptr(prep["QL"]), _lib.ptr(m), _lib.ptr(c))

            def one():
                m.copy_(m0)
                if prec == "float64":
                    rc = lib.pof_ieks_solve(_lib.POF_F64, n, D, d, int(prep["fields"][b]), *args_c, maxiters, 1,
                                            _lib.ptr(inf), _lib.ptr(ws), wsb, _lib.stream_handle())
                else:
                    rc = lib.pof_ieks_solve_mixed(n, D, d, int(prep["fields"][b]), *args_c, maxiters, 1e-5,
                                                  args.f32_settle, maxiters, 1, _lib.ptr(inf), _lib.ptr(ws), wsb,
                                                  _lib.stream_handle())
                _lib.check(rc, "solve")

            ms = timed(one)
            per.append({"ms": ms, "iterations": int(inf[_lib.I_ITERATIONS].item()),
                        "iterations_float32": int(inf[_lib.I_COUNT].item()) if prec == "mixed" else 0,
                        "best_change_float32": float(inf[_lib.I_COUNT + 1].item()) if prec == "mixed" else None,
                        "y": m[:, ::q + 1].clone()})
        results["plain_" + prec] = per
    ref = [r["y"] for r in results["plain_float64"]]
    # batched, float64 and mixed
    means = torch.empty_like(prep["means0"])
    G = means.shape[0]
    chols = torch.empty((G, D, D), dtype=torch.float64, device=dev)
    info = torch.zeros((B, _lib.I_COUNT), dtype=torch.float64, device=dev)
    info32 = torch.zeros((B, 2), dtype=torch.float64, device=dev)
    for prec in ("float64", "mixed"):
        ws = [None]

        def one():
            means.copy_(prep["means0"])
            ws[0] = pbatch.run_batch(prep, means, chols, info, maxiters=maxiters, workspace=ws[0], precision=prec,
                                     maxiters_f32=maxiters, info_f32=info32, settle_f32=args.f32_settle)

        ms = timed(one)
        ys = [means[off[b]:off[b + 1], ::q + 1] for b in range(B)]
        results["batched_" + prec] = {"ms": ms, "y": ys, "iterations": info[:, _lib.I_ITERATIONS].tolist(),
                                      "iterations_float32": info32[:, 0].tolist() if prec == "mixed" else None,
                                      "best_change_float32": info32[:, 1].tolist() if prec == "mixed" else None}

    def err(y, r):
        return float(((y - r).abs().max() / r.abs().max()).item())

    names = ["%s%s" % (nm, p) for (nm, p, _, _) in spec]
    out_probs = []
    for b in range(B):
        pf, pm = results["plain_float64"][b], results["plain_mixed"][b]
        out_probs.append({
            "problem": names[b], "N": N, "q": q,
            "plain_float64": {"ms": pf["ms"], "iterations": pf["iterations"]},
            "plain_mixed": {"ms": pm["ms"], "iterations_float64": pm["iterations"],
                            "iterations_float32": pm["iterations_float32"],
                            "best_change_float32": pm["best_change_float32"], "max_rel_err": err(pm["y"], ref[b])},
            "batched_mixed_max_rel_err": err(results["batched_mixed"]["y"][b], ref[b]),
            "batched_float64_max_rel_err": err(results["batched_float64"]["y"][b], ref[b]),
        })
    plain64_ms = sum(r["ms"] for r in results["plain_float64"])
    plainmx_ms = sum(r["ms"] for r in results["plain_mixed"])
    if rank != 0:
        return
    jprint({
        "metric": "IVP*steps/s, mixed precision (float32 iterations + float64 polish) vs float64",
        "value": steps / (results["batched_mixed"]["ms"] * 1e-3),
        "unit": "IVP*steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": results["batched_mixed"]["ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": workload, "problems": names, "N": N, "q": q, "D": D, "maxiters": maxiters,
                   "omitted": "the reaction-diffusion system (d = 128) of the configuration: its mixed solve runs "
                              "on the dense path from the host (--workload rd_d640 --dense-solve)"},
        "plain_float64": {"value": steps / (plain64_ms * 1e-3), "ms": plain64_ms},
        "plain_mixed": {"value": steps / (plainmx_ms * 1e-3), "ms": plainmx_ms},
        "batched_float64": {"value": steps / (results["batched_float64"]["ms"] * 1e-3),
                            "ms": results["batched_float64"]["ms"], "iterations": results["batched_float64"]["iterations"]},
        "batched_mixed": {"value": steps / (results["batched_mixed"]["ms"] * 1e-3), "ms": results["batched_mixed"]["ms"],
                          "iterations_float64": results["batched_mixed"]["iterations"],
                          "iterations_float32": results["batched_mixed"]["iterations_float32"],
                          "best_change_float32": results["batched_mixed"]["best_change_float32"]},
        "speedup_batched_mixed_vs_plain_float64": plain64_ms / results["batched_mixed"]["ms"],
        "problems": out_probs,
    })


DENSE_WORKLOADS = {
    # name: (cells, q, N, tmax): the method-of-lines FitzHugh-Nagumo
    # reaction-diffusion system (pof.ivp.fhn_reaction_diffusion: 64 periodic
    # cells, d = 128, D = 640 at q = 4), uniform grid of N points
    "rd_d640": (64, 4, 2 ** 12, 20.0),
}


def dense_passes(workload, precisions, f64_steps, steps, warmup, n_override=0):
    """Time one IEKS iteration's work on the dense path (EK1 linearization of
    the reaction-diffusion field + the dense filter + smoother pass) from the
    constant-init trajectory: float32 over the whole grid, float64 over its
    first f64_steps steps (the per-step cost is uniform: the chunks run their
    steps one after the other, the tree above them adds log2(P) levels).
    Returns {precision: {...}} and the problem's set-up."""
    import torch

    from pof import _flops, ivp as pivp
    from pof.convenience import get_initial_trajectory, set_up_solver
    from pof.parallel_filtsmooth import linear_filtsmooth
    from pof.step import linearize_at_previous_states
    from pof.utils import MVNSqrt

    cells, q, N, tmax = DENSE_WORKLOADS[workload]
    if n_override:
        N = n_override
    pv = pivp.fhn_reaction_diffusion(cells=cells, tmax=tmax)
    ts = torch.linspace(0.0, tmax, N, dtype=torch.float64)
    setup = set_up_solver(f=pv.f, y0=pv.y0, ts=ts, order=q)
    states = get_initial_trajectory(setup, method="constant")
    D = states.mean.shape[1]
    d = 2 * cells
    n = N - 1
    env_chunks = int(os.environ.get("POF_DENSE_CHUNKS", "0"))
    x0, dtm = setup["x0"], setup["dtm"]

    def timed(fn):
        for _ in range(warmup):
            fn()
        ts_ = []
        for _ in range(steps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            ts_.append(e0.elapsed_time(e1))
        return float(np.median(ts_))

    out = {}
    passes = [("float32", n), ("float64", min(n, f64_steps))]
    for prec, nsteps in [pp for pp in passes if pp[0] in precisions]:
        dt = torch.float32 if prec == "float32" else torch.float64
        sub = MVNSqrt(states.mean[: nsteps + 1], states.chol[: nsteps + 1])
        F, QL = dtm.F[0].to(dt), dtm.QL[0].to(dt)
        x0t = MVNSqrt(x0.mean.to(dt), x0.chol.to(dt))
        res = {}

        def one():
            dom = linearize_at_previous_states(setup["om"], sub)
            res["out"] = linear_filtsmooth(x0t, (F, QL), (dom.H.to(dt), dom.b.to(dt), None))

        ms = timed(one)
        chunks = min(env_chunks or (256 if prec == "float32" else 64), nsteps)
        fl = _flops.dense_pass_flops(nsteps, D, d, chunks)
        out[prec] = {"steps": nsteps, "chunks": chunks, "ms_per_pass": ms, "ms_per_step": ms / nsteps,
                     "gflops": fl / (ms * 1e-3) / 1e9, "flop_model_tflop": fl / 1e12,
                     "finite": bool(torch.isfinite(res["out"][0].mean).all().item())}
        del res
    info = {"cells": cells, "d": d, "D": D, "q": q, "N": N, "tmax": tmax,
            "field_params": "a = b = 0.2, c = 3, kv = 0.5, kw = 0.05, v0 = -1 + 0.5 sin(2 pi k / 64), w0 = 1"}
    return out, info, (pv, ts, q)


def dense_block(args):
    """The default line's dense block: the reaction-diffusion system at
    (D, d) = (640, 128), N = 2^12 -- a float32 pass over the whole grid and a
    float64 pass over its first 256 steps (one IEKS iteration's work each)."""
    import torch

    from pof import _lib

    out, info, setup = dense_passes("rd_d640", ("float32", "float64"), 256, 1, 1)
    peak64 = fp64_peak(torch, _lib.lib(), _lib)
    out["float64"]["frac_of_fp64_probe"] = out["float64"]["gflops"] / peak64
    torch.cuda.empty_cache()
    try:
        cpu = dense_cpu_sample(setup, 4)
    except Exception as e:  # noqa: BLE001
        cpu = {"error": "%s: %s" % (type(e).__name__, e), "ms_per_step": None}
    return {"workload": "rd_d640: method-of-lines FitzHugh-Nagumo, 64 periodic cells (d = 128), q = 4 (D = 640), "
                        "N = 4096, t in [0, 20]; one IEKS iteration's work (EK1 + dense filter + smoother) from "
                        "the constant-init trajectory; float64 over the first 256 steps",
            "config": info, "float32": out["float32"], "float64": out["float64"], "fp64_probe_gflops": peak64,
            "flop_model": "pof/_flops.py dense_pass_flops: 12.3 GFLOP per step at (640, 128)",
            "cpu_baseline": cpu,
            "float64_vs_cpu_per_step": (cpu["ms_per_step"] / out["float64"]["ms_per_step"]
                                        if cpu.get("ms_per_step") else None)}


def dense_cpu_sample(setup, nsteps):
    """One IEKS iteration of the reference's algorithm restated in NumPy
    float64 (the oracle: EK1 linearization at the constant-init trajectory,
    then the associative-scan filter + smoother of
    oracle.filtsmooth.linear_filtsmooth) on the first `nsteps` steps of the
    dense workload's grid, on this host's cores (NumPy's BLAS/LAPACK
    threads): ms per step."""
    from oracle import filtsmooth as ofs, ivp as oivp, solver as osolver

    pv, ts, q = setup
    cells = pv.y0.shape[0] // 2
    o = oivp.fhn_reaction_diffusion(cells=cells, tmax=float(ts[-1]))
    grid = np.asarray(ts[: nsteps + 1], dtype=np.float64)
    st = osolver.set_up_solver(o, grid, q)
    states = osolver.get_initial_trajectory(st, "constant")
    t0 = time.perf_counter()
    dom = osolver.linearize_at_previous_states(st, states[0])
    ofs.linear_filtsmooth(st.x0, (st.F, st.QL), dom)
    sec = time.perf_counter() - t0
    return {"value": sec * 1e3 / nsteps, "ms_per_step": sec * 1e3 / nsteps, "unit": "ms per step (one IEKS iteration)",
            "kind": "port", "cores": os.cpu_count(),
            "sample": "the oracle (the reference's algorithm in NumPy float64): EK1 at the constant-init trajectory "
                      "and the associative-scan filter + smoother on the first %d steps of the same grid (set-up not "
                      "timed), NumPy's BLAS/LAPACK threads on this host" % nsteps}


def run_dense(args, workload):
    """The dense workload on its own line (python bench.py --workload rd_d640);
    with --dense-solve also the whole mixed-precision solve (float32
    iterations, float64 polish)."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from pof import _build, _lib, solver as psolver

    _build.build(verbose=False)
    lib = _lib.lib()
    out, info, (pv, ts, q) = dense_passes(workload, args.dense_precisions.split(","), args.dense_f64_steps,
                                          args.steps, args.warmup, args.dense_n)
    peak64 = fp64_peak(torch, lib, _lib)
    n = info["N"] - 1
    full64_ms = None
    if "float64" in out:
        out["float64"]["frac_of_fp64_probe"] = out["float64"]["gflops"] / peak64
        full64_ms = out["float64"]["ms_per_step"] * n
    solve = None
    if args.dense_solve:
        t0 = time.time()
        # bounded: at most 30 float32 and 5 + 1 float64 iterations (~57 s each at
        # (640, 128), N = 4096); the status says whether it converged
        (ym, yL), sinfo = psolver.solve(f=pv.f, y0=pv.y0, ts=ts, order=q, init="constant", precision="mixed",
                                        rtol_f32=1e-4, maxiters=5, maxiters_f32=30)
        torch.cuda.synchronize()
        solve = {"seconds": time.time() - t0, "iterations_float32": int(sinfo["iterations_float32"]),
                 "iterations_float64": int(sinfo["iterations"]), "status": int(sinfo["status"])}
    if rank != 0:
        return
    first = next(iter(out.values()))
    jprint({
        "metric": "dense filter + smoother pass (one IEKS iteration's work), ms per pass",
        "value": first["ms_per_pass"], "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": first["ms_per_pass"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (value), f64", "data": "synthetic",
        "config": dict(info, workload=workload),
        "float32": out.get("float32"), "float64": out.get("float64"),
        "float64_full_grid_ms_estimate": full64_ms, "fp64_probe_gflops": peak64, "mixed_solve": solve,
    })


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD,
                    choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS) + sorted(SERVE_WORKLOADS)
                    + sorted(MIXED_WORKLOADS) + sorted(SWEEP_WORKLOADS) + sorted(DENSE_WORKLOADS))
    ap.add_argument("--dense-n", type=int, default=0, help="grid points of the dense workload (0: its own)")
    ap.add_argument("--dense-f64-steps", type=int, default=256,
                    help="steps of the float64 pass of the dense workload")
    ap.add_argument("--dense-solve", action="store_true",
                    help="also run the dense workload's mixed solve (bounded: 30 float32 + 6 float64 iterations)")
    ap.add_argument("--dense-precisions", default="float32,float64", help="passes of the dense workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default line without its config0 / batched / served blocks")
    ap.add_argument("--f32-settle", type=float, default=0.1,
                    help="mixed precision: count non-shrinking float32 changes only once the smallest change is "
                         "below this (inf: from the first iteration, the library's default)")
    ap.add_argument("--solves-only", action="store_true",
                    help="run the W + K solves of the workload and exit (for profiler captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args, args.workload)
    elif args.workload in BATCH_WORKLOADS:
        run_gpu_batch(args, args.workload)
    elif args.workload in SERVE_WORKLOADS:
        run_serve(args, args.workload)
    elif args.workload in MIXED_WORKLOADS:
        run_mixed(args, args.workload)
    elif args.workload in SWEEP_WORKLOADS:
        run_sweep(args, args.workload)
    elif args.workload in DENSE_WORKLOADS:
        run_dense(args, args.workload)
    else:
        run_gpu(args, args.workload)


if __name__ == "__main__":
    main()
