"""Continuous-batching IEKS server (no counterpart in the reference, which
solves one IVP per ``pof.solver.solve`` call, pof/solver.py:11-73).

Requests -- (field name, params, y0, ts) with a built-in field, an order q,
an objective tolerance and maxiters -- are queued on the host and admitted
into one libpof engine per state shape (D, d) as request slots and memory
free up.  Every tick runs one IEKS iteration of every admitted, unfinished
request; requests that meet their criterion leave at once and their result
is fetched.  Engines of different shapes run on their own CUDA streams, so
their work overlaps on the device.  A request's result is bit-identical to
the same request served alone (pof_server_* in include/pof.h).
"""

import ctypes
import threading
import time
from collections import deque
from typing import Any, NamedTuple

import numpy as np
import torch

from . import _lib
from . import batch as pbatch
from .transitions import IWP, preconditioned_discretize
from .utils import default_device


class Request(NamedTuple):
    rid: int
    field: str
    params: tuple
    y0: Any
    ts: Any
    order: int
    rtol: float
    maxiters: int
    deadline: float = float("inf")  # perf_counter time after which the request is cancelled


class Engine:
    """One libpof engine: requests of state shape (D, d) = (d (q+1), d)."""

    def __init__(self, d, q, max_requests, max_points, level_bytes=None, device=None, calibrate=True,
                 precision="float64", maxiters_f32=10_000, rtol_f32=1e-5, settle_f32=float("inf")):
        self.dev = device or default_device()
        self.d, self.q = d, q
        self.D = d * (q + 1)
        self.mixed = precision == "mixed"
        if precision not in ("float64", "mixed"):
            raise ValueError("precision must be 'float64' or 'mixed'")
        lib = _lib.lib()
        if level_bytes is None:  # scan levels for chunks of >= 4 steps (about 56 D^2 bytes per chunk, x 2)
            level_bytes = 28 * self.D * self.D * max_points + (64 << 20)
        query = lib.pof_server_mixed_workspace_bytes if self.mixed else lib.pof_server_workspace_bytes
        wsb = query(self.D, d, max_requests, max_points, int(level_bytes))
        if wsb == 0:
            raise _lib.PofError("no batched kernels for (D, d) = (%d, %d)" % (self.D, d))
        self.ws = _lib.workspace(wsb, self.dev)
        F, QL = preconditioned_discretize(IWP(num_derivatives=q, wiener_process_dimension=d), device=self.dev)
        self.F, self.QL = F.contiguous(), QL.contiguous()
        h = ctypes.c_void_p()
        if self.mixed:
            settle = min(float(settle_f32), 1e300)
            _lib.check(lib.pof_server_create_mixed(self.D, d, max_requests, max_points, int(level_bytes),
                                                   _lib.ptr(self.F), _lib.ptr(self.QL), int(bool(calibrate)),
                                                   int(maxiters_f32), float(rtol_f32), settle, _lib.ptr(self.ws),
                                                   int(wsb), ctypes.byref(h)), "pof_server_create_mixed")
        else:
            _lib.check(lib.pof_server_create(self.D, d, max_requests, max_points, int(level_bytes),
                                             _lib.ptr(self.F), _lib.ptr(self.QL), int(bool(calibrate)),
                                             _lib.ptr(self.ws), int(wsb), ctypes.byref(h)), "pof_server_create")
        self.h = h
        self.slots = {}  # slot -> (request, p0)
        self.running = 0

    def close(self):
        if self.h:
            _lib.lib().pof_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, req, x0m, row, h, p0):
        """Admit a prepared request; False when the engine is full."""
        lib = _lib.lib()
        prm = np.zeros(4, dtype=np.float64)
        prm[: len(req.params)] = req.params
        x0m = np.ascontiguousarray(x0m, dtype=np.float64)
        row = np.ascontiguousarray(row, dtype=np.float64)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        slot = lib.pof_server_submit(self.h, len(req.ts) - 1, _lib.FIELDS[req.field], vp(prm), float(h), vp(x0m),
                                     None, vp(row), int(req.maxiters), float(req.rtol))
        if slot == _lib.POF_ERR_BUSY:
            return False
        if slot < 0:
            _lib.check(int(slot), "pof_server_submit")
        self.slots[int(slot)] = (req, p0)
        return True

    def cancel(self, rid):
        """Set the engine's cancel flag of request rid (admitted, unfinished):
        it stops at the engine's next tick with status "cancelled" and its
        last iterate, and is collected by finished() like any other.  False
        when rid is not in this engine."""
        for slot, (req, _) in self.slots.items():
            if req.rid == rid:
                _lib.check(_lib.lib().pof_server_cancel(self.h, int(slot)), "pof_server_cancel")
                return True
        return False

    def launch(self, k=1):
        _lib.check(_lib.lib().pof_server_launch(self.h, int(k)), "pof_server_launch")

    def sync(self):
        n = ctypes.c_int64(0)
        _lib.check(_lib.lib().pof_server_sync(self.h, ctypes.byref(n)), "pof_server_sync")
        self.running = n.value
        return self.running

    def finished(self):
        """[(request, (means, chols), info)] of the requests that finished since the last call."""
        lib = _lib.lib()
        out = []
        buf = (ctypes.c_int64 * 256)()
        while True:
            n = lib.pof_server_poll(self.h, ctypes.cast(buf, ctypes.c_void_p), 256)
            if n <= 0:
                break
            for i in range(n):
                slot = int(buf[i])
                req, p0 = self.slots.pop(slot)
                N = len(req.ts)
                m = torch.empty((N, self.D), dtype=torch.float64, device=self.dev)
                L = torch.empty((N, self.D, self.D), dtype=torch.float64, device=self.dev)
                info = torch.empty(_lib.I_COUNT + (2 if self.mixed else 0), dtype=torch.float64, device=self.dev)
                if self.mixed:  # float32 iterations kept, smallest float32 change (before the slot is freed)
                    _lib.check(lib.pof_server_mixed_info(self.h, slot, _lib.ptr(info[_lib.I_COUNT:])),
                               "pof_server_mixed_info")
                _lib.check(lib.pof_server_fetch(self.h, slot, _lib.ptr(m), _lib.ptr(L), _lib.ptr(info)),
                           "pof_server_fetch")
                idx = torch.arange(self.d, device=self.dev) * (self.q + 1)
                ys = (m[:, idx] * p0, L[:, idx, :] * p0)
                out.append((req, ys, info))
            if n < 256:
                break
        return out


def dense_field(field, params, y0):
    """The torch vector field of a request for a field the dense path solves
    (pof._lib.DENSE_FIELDS)."""
    from . import ivp as pivp

    if field == "fhn_rd":
        a, b, c, kv, kw = (float(p) for p in params)
        return pivp.fhn_reaction_diffusion(cells=len(y0) // 2, a=a, b=b, c=c, kv=kv, kw=kw, y0=y0).f
    raise ValueError("no dense field %r" % (field,))


class _DenseJob:
    def __init__(self, req, nbytes):
        self.req = req
        self.nbytes = nbytes
        self.stop = threading.Event()
        self.out = None
        self.error = None
        self.thread = None


class DenseLane:
    """Requests of the dense path's fields (state dimension D >= 32, e.g. the
    reaction-diffusion system of pof.ivp.fhn_reaction_diffusion): each
    admitted request runs its IEKS loop (pof.solver.solve, the host-driven
    loop over the dense filter/smoother) on a CUDA stream of its own in a
    worker thread, so its kernels overlap with the serving engines' and with
    the other dense requests'.  Admission in arrival order while the sum of
    the running requests' memory (dense workspace, trajectories, linearized
    models) stays within budget_bytes; cancellation and timeouts act before
    the request's next IEKS iteration.  A request's result is the one
    pof.solver.solve gives for it alone."""

    def __init__(self, device, budget_bytes, precision="float64", maxiters_f32=10_000, rtol_f32=1e-5,
                 settle_f32=float("inf"), solve=None):
        self.dev = device
        self.budget = int(budget_bytes)
        self.precision = dict(precision=precision, maxiters_f32=maxiters_f32, rtol_f32=rtol_f32,
                              settle_f32=settle_f32)
        self.jobs = {}  # rid -> _DenseJob
        self._solve = solve

    def bytes_for(self, req):
        """Device memory of one request: the dense workspace (float64, and
        float32 for mixed precision), three trajectories and the linearized
        model."""
        lib = _lib.lib()
        d = len(req.y0)
        D = d * (req.order + 1)
        n = len(req.ts) - 1
        ws = lib.pof_dense_workspace_bytes(_lib.POF_F64, 1, n, D, d, 0)
        if self.precision["precision"] == "mixed":
            ws += lib.pof_dense_workspace_bytes(_lib.POF_F32, 1, n, D, d, 0)
        return int(ws + 3 * 8 * (n + 1) * D * (D + 1) + 2 * 8 * n * d * (D + d))

    def in_use(self):
        return sum(j.nbytes for j in self.jobs.values())

    def submit(self, req):
        """Start request req if the budget allows (the first request always
        starts); False otherwise."""
        nb = self.bytes_for(req)
        if self.jobs and self.in_use() + nb > self.budget:
            return False
        job = _DenseJob(req, nb)
        job.thread = threading.Thread(target=self._run, args=(job,), daemon=True)
        self.jobs[req.rid] = job
        job.thread.start()
        return True

    def _run(self, job):
        req = job.req
        try:
            if self._solve is not None:  # a stand-in for tests without a GPU
                job.out = self._solve(req, job.stop.is_set)
                return
            from . import solver

            torch.cuda.set_device(self.dev)
            st = torch.cuda.Stream(self.dev)
            with torch.cuda.stream(st):
                f = dense_field(req.field, req.params, torch.as_tensor(req.y0, dtype=torch.float64))
                ys, info = solver.solve(f=f, y0=torch.as_tensor(req.y0, dtype=torch.float64),
                                        ts=torch.as_tensor(req.ts, dtype=torch.float64), order=req.order,
                                        init="constant", maxiters=req.maxiters, rtol=req.rtol,
                                        stop=job.stop.is_set, **self.precision)
                st.synchronize()
            job.out = (ys, info)
        except Exception as e:  # reported by finished()
            job.error = e

    def cancel(self, rid):
        job = self.jobs.get(rid)
        if job is None:
            return False
        job.stop.set()
        return True

    def finished(self):
        """[(request, (means, chols), info tensor)] of the requests whose
        loop ended since the last call."""
        out = []
        for rid in [r for r, j in self.jobs.items() if not j.thread.is_alive()]:
            job = self.jobs.pop(rid)
            if job.error is not None:
                raise job.error
            ys, info = job.out
            t = torch.zeros(_lib.I_COUNT + (2 if "iterations_float32" in info else 0), dtype=torch.float64)
            t[_lib.I_ITERATIONS] = float(info["iterations"])
            t[_lib.I_NLL] = float(info["nll"])
            t[_lib.I_OBJ] = float(info["obj"])
            t[_lib.I_SSQ] = float(info["sigma_squared"])
            t[_lib.I_STATUS] = float(info["status"])
            if "iterations_float32" in info:
                t[_lib.I_COUNT] = float(info["iterations_float32"])
                t[_lib.I_COUNT + 1] = float(info["best_change_float32"])
            out.append((job.req, (ys.mean, ys.chol), t))
        return out

    def close(self):
        for job in self.jobs.values():
            job.stop.set()
        for job in self.jobs.values():
            job.thread.join()
        self.jobs = {}


class Server:
    """Host side of continuous batching: a FIFO of requests, one Engine per
    (d, q), admission each tick as memory allows; requests of the dense
    path's fields go to the DenseLane (dense_budget_bytes of device memory
    for the running ones)."""

    def __init__(self, max_requests=1024, max_points=1 << 21, device=None, precision="float64", maxiters_f32=10_000,
                 rtol_f32=1e-5, settle_f32=float("inf"), dense_budget_bytes=64 << 30, dense_solve=None):
        """precision="mixed": every request runs float32 IEKS iterations first
        and float64 ones after (pof_server_create_mixed; the float32 phase's
        rules and discard rule are those of pof.solver.solve's
        precision="mixed")."""
        self.dev = device or default_device()
        self.max_requests = max_requests
        self.max_points = max_points
        self.precision = dict(precision=precision, maxiters_f32=maxiters_f32, rtol_f32=rtol_f32,
                              settle_f32=settle_f32)
        self.engines = {}
        self.queue = deque()
        self.results = {}
        self.next_rid = 0
        self.t_submit = {}
        self.t_done = {}
        self.prepared = {}
        self.stop_reason = {}  # rid -> "cancelled" | "timeout" for requests stopped by the host
        self.dense = DenseLane(self.dev, dense_budget_bytes, solve=dense_solve, **self.precision)
        self.dense_queue = deque()

    def engine(self, d, q):
        key = (d, q)
        if key not in self.engines:
            self.engines[key] = Engine(d, q, self.max_requests, self.max_points, device=self.dev, **self.precision)
        return self.engines[key]

    def submit(self, field, params, y0, ts, order, rtol=1e-6, maxiters=10_000, t_arrival=None, timeout=None):
        """Queue a request; returns its id.  timeout (seconds from arrival):
        a request still unfinished then is cancelled -- taken out of the queue,
        or stopped by its engine at the next tick -- and reported with status
        "timeout"."""
        rid = self.next_rid
        self.next_rid += 1
        t0 = time.perf_counter() if t_arrival is None else t_arrival
        deadline = float("inf") if timeout is None else t0 + float(timeout)
        req = Request(rid, field, tuple(float(p) for p in params), np.asarray(y0, dtype=np.float64),
                      np.asarray(ts, dtype=np.float64), int(order), float(rtol), int(maxiters), deadline)
        (self.dense_queue if field in _lib.DENSE_FIELDS else self.queue).append(req)
        self.t_submit[rid] = t0
        return rid

    def cancel(self, rid, reason="cancelled"):
        """Stop request rid: a queued one leaves the queue at once (its
        result is (None, info) with no iterations); an admitted one stops at
        its engine's next tick with its last iterate.  Either way its status
        is `reason`.  False when rid has already finished."""
        if rid in self.results:
            return False
        for r in list(self.queue) + list(self.dense_queue):
            if r.rid == rid:
                self.queue = deque(q for q in self.queue if q.rid != rid)
                self.dense_queue = deque(q for q in self.dense_queue if q.rid != rid)
                self.prepared.pop(rid, None)
                info = torch.full((_lib.I_COUNT,), float("nan"), dtype=torch.float64)
                info[_lib.I_ITERATIONS] = 0.0
                info[_lib.I_STATUS] = 3.0  # POF_SOLVE_CANCELLED
                self.results[rid] = (None, info)
                self.t_done[rid] = time.perf_counter()
                self.stop_reason[rid] = reason
                return True
        for e in self.engines.values():
            if e.cancel(rid):
                self.stop_reason[rid] = reason
                return True
        if self.dense.cancel(rid):
            self.stop_reason[rid] = reason
            return True
        return False

    def _expire(self):
        """Cancel the requests whose deadline has passed (status "timeout")."""
        now = time.perf_counter()
        late = [r.rid for r in list(self.queue) + list(self.dense_queue) if r.deadline <= now]
        for e in self.engines.values():
            late += [req.rid for req, _ in e.slots.values() if req.deadline <= now and req.rid not in self.stop_reason]
        late += [rid for rid, j in self.dense.jobs.items() if j.req.deadline <= now and rid not in self.stop_reason]
        for rid in late:
            self.cancel(rid, reason="timeout")

    def _admit(self):
        """Prepare and admit queued requests in arrival order while engines take them."""
        while self.dense_queue and self.dense.submit(self.dense_queue[0]):
            self.dense_queue.popleft()
        if not self.queue:
            return
        reqs = list(self.queue)
        groups = {}
        for r in reqs:
            if r.rid not in self.prepared:
                groups.setdefault((pbatch._DIM[r.field], r.order), []).append(r)
        for (d, q), rs in groups.items():
            prep = pbatch.prepare_rows([(r.field, r.params, r.y0, r.ts) for r in rs], q)
            for i, r in enumerate(rs):
                self.prepared[r.rid] = (prep["x0m"][i].numpy(), prep["row"][i].numpy(), float(prep["h"][i]),
                                        float(prep["p0"][i]))
        prepared = self.prepared
        kept = deque()
        blocked = set()
        for r in reqs:
            key = (pbatch._DIM[r.field], r.order)
            if key in blocked:
                kept.append(r)
                continue
            x0m, row, h, p0 = prepared[r.rid]
            if self.engine(*key).submit(r, x0m, row, h, p0):
                del prepared[r.rid]
            else:
                blocked.add(key)  # keep FIFO order within a shape
                kept.append(r)
        self.queue = kept

    def tick(self, k=1):
        """Cancel what is past its deadline, admit, run k iterations on every
        engine (overlapping), collect the finished requests; returns their
        ids."""
        self._expire()
        self._admit()
        live = [e for e in self.engines.values() if e.slots]
        for e in live:
            e.launch(k)
        done = []
        for e in live:
            e.sync()
            for req, ys, info in e.finished():
                self.results[req.rid] = (ys, info)
                self.t_done[req.rid] = time.perf_counter()
                done.append(req.rid)
        for req, ys, info in self.dense.finished():
            self.results[req.rid] = (ys, info)
            self.t_done[req.rid] = time.perf_counter()
            done.append(req.rid)
        return done

    def busy(self):
        return (bool(self.queue) or bool(self.dense_queue) or bool(self.dense.jobs)
                or any(e.slots for e in self.engines.values()))

    def result(self, rid):
        """((means (N, d), chol_covs (N, d, D)), info) as pof.solver.solve
        returns, with info["status"] the request's outcome: "converged",
        "maxiters", "nonfinite" (NaN or infinite objective: a poisoned input),
        "cancelled" or "timeout".  A request cancelled before admission has
        no result (None)."""
        ys, info = self.results[rid]
        status = _lib.solve_status(float(info[_lib.I_STATUS]))
        if status == "cancelled":
            status = self.stop_reason.get(rid, status)
        out = {"iterations": info[_lib.I_ITERATIONS].to(torch.int64), "nll": info[_lib.I_NLL],
               "obj": info[_lib.I_OBJ], "sigma_squared": info[_lib.I_SSQ], "status": status, "calibrated": True}
        if info.shape[0] > _lib.I_COUNT:  # a mixed-precision engine's request
            out["iterations_float32"] = info[_lib.I_COUNT].to(torch.int64)
            out["best_change_float32"] = info[_lib.I_COUNT + 1]
        return ys, out

    def close(self):
        self.dense.close()
        for e in self.engines.values():
            e.close()
        self.engines = {}
