"""Host side of the continuous-batching server (pof.serve) on CPU.

`pof.serve.Server` queues requests, keeps one engine per (d, q), admits
requests in arrival order while an engine has a free slot and memory, runs
ticks and collects finished requests.  Here libpof's engine (pof_server_*,
which the GPU tests exercise) is replaced by a host fake with the same
contract: a slot table, a grid-point budget, and requests that finish after
a number of iterations fixed at admission.  The tests check the Server's
own logic: FIFO admission within a shape, shapes that do not block one
another, queueing under the memory budget, and the results each request
gets back.
"""

import ctypes
import threading
import time

import numpy as np
import pytest
import torch

from pof import _lib, batch as pbatch, serve
from pof.utils import MVNSqrt

CPU = torch.device("cpu")
BUSY = -7


class FakeEngines:
    """pof_server_* on the host.  A request of n steps holds n + 1 grid
    points from admission until its result is fetched, and finishes after
    `iterations(n)` IEKS iterations."""

    def __init__(self, iterations):
        self.iterations = iterations
        self.servers = {}
        self.log = []  # (event, engine (D, d), slot, n_steps)

    def _s(self, h):
        return self.servers[h.value if isinstance(h, ctypes.c_void_p) else h]

    def pof_status_string(self, rc):
        return b"fake status %d" % rc

    def pof_server_workspace_bytes(self, D, d, max_requests, max_points, level_bytes):
        return 4096

    def pof_server_create(self, D, d, max_requests, max_points, level_bytes, F, QL, calibrate, ws, wsb, out):
        h = len(self.servers) + 1
        self.servers[h] = {"D": D, "d": d, "maxB": max_requests, "maxG": max_points, "used": 0, "slots": {},
                           "done": []}
        out._obj.value = h
        return 0

    def pof_server_destroy(self, h):
        return 0

    def pof_server_mixed_workspace_bytes(self, D, d, max_requests, max_points, level_bytes):
        return 8192

    def pof_server_create_mixed(self, D, d, max_requests, max_points, level_bytes, F, QL, calibrate, maxiters_f32,
                                rtol_f32, settle_f32, ws, wsb, out):
        rc = self.pof_server_create(D, d, max_requests, max_points, level_bytes, F, QL, calibrate, ws, wsb, out)
        self.servers[out._obj.value].update(mixed=(maxiters_f32, rtol_f32, settle_f32))
        return rc

    def pof_server_mixed_info(self, h, slot, info):
        s = self._s(h)
        r = s["slots"][slot]
        a = np.array([r["n"] % 7 + 1.0, 1e-6])  # a stand-in float32 count per request
        ctypes.memmove(info.value, a.ctypes.data, a.nbytes)
        return 0

    def pof_server_submit(self, h, n_steps, field, params, step, x0m, x0L, row, maxiters, rtol):
        s = self._s(h)
        free = [i for i in range(s["maxB"]) if i not in s["slots"]]
        if not free or s["used"] + n_steps + 1 > s["maxG"]:
            return BUSY
        slot = free[0]
        s["slots"][slot] = {"n": n_steps, "it": 0, "target": self.iterations(n_steps), "done": False,
                            "cancel": False, "status": 0}
        s["used"] += n_steps + 1
        self.log.append(("admit", (s["D"], s["d"]), slot, n_steps))
        return slot

    def pof_server_launch(self, h, k):
        s = self._s(h)
        for slot, r in sorted(s["slots"].items()):
            for _ in range(k):
                if r["done"]:
                    break
                r["it"] += 1
                if r["cancel"] or r["it"] >= r["target"]:
                    # a cancelled request stops at the first tick after the flag
                    r["status"] = 3 if (r["cancel"] and r["it"] < r["target"]) else 0
                    r["done"] = True
                    s["done"].append(slot)
        return 0

    def pof_server_cancel(self, h, slot):
        s = self._s(h)
        r = s["slots"].get(slot)
        if r is None or r["done"]:
            return -1
        r["cancel"] = True
        self.log.append(("cancel", (s["D"], s["d"]), slot, r["n"]))
        return 0

    def pof_server_sync(self, h, nref):
        nref._obj.value = sum(1 for r in self._s(h)["slots"].values() if not r["done"])
        return 0

    def pof_server_poll(self, h, buf, cap):
        s = self._s(h)
        out, s["done"] = s["done"][:cap], s["done"][cap:]
        arr = (ctypes.c_int64 * cap).from_address(buf.value)
        for i, slot in enumerate(out):
            arr[i] = slot
        return len(out)

    def pof_dense_workspace_bytes(self, dtype, which, n, D, d, chunks):
        return 1000 * n

    def pof_server_fetch(self, h, slot, m, L, info):
        s = self._s(h)
        r = s["slots"].pop(slot)
        s["used"] -= r["n"] + 1
        N, D = r["n"] + 1, s["D"]
        # every state's mean holds (n_steps, slot) so the test can tell results apart
        mean = np.tile(np.array([r["n"], slot] * D, dtype=np.float64)[:D], (N, 1))
        chol = np.zeros((N, D, D))
        inf = np.array([r["it"], 1.0, 2.0, 3.0, r["status"]])
        for ptr, a in ((m, mean), (L, chol), (info, inf)):
            ctypes.memmove(ptr.value, a.ctypes.data, a.nbytes)
        self.log.append(("fetch", (s["D"], s["d"]), slot, r["n"]))
        return 0


@pytest.fixture
def fake(monkeypatch):
    f = FakeEngines(iterations=lambda n: 2 + n // 100)
    monkeypatch.setattr(_lib, "lib", lambda: f)
    # the fake engine takes host tensors (the real pointer helper refuses them)
    monkeypatch.setattr(_lib, "ptr", lambda t: None if t is None else ctypes.c_void_p(t.data_ptr()))
    monkeypatch.setattr(serve, "default_device", lambda: CPU)
    return f


def _run(srv, limit=1000):
    ticks = 0
    while srv.busy():
        srv.tick()
        ticks += 1
        assert ticks < limit
    return ticks


def logistic(n):
    return ("logistic", (3.0,), [0.01], np.linspace(0.0, 10.0, n + 1))


def vdp(n):
    return ("vanderpol", (1.0,), [2.0, 0.0], np.linspace(0.0, 6.3, n + 1))


def test_fifo_admission_with_two_slots(fake):
    srv = serve.Server(max_requests=2, max_points=10**6)
    ns = [450, 120, 300, 50, 220]
    rids = [srv.submit(*logistic(n), order=2) for n in ns]
    _run(srv)
    admitted = [n for ev, _, _, n in fake.log if ev == "admit"]
    assert admitted == ns  # arrival order
    live = 0
    for ev, _, _, _ in fake.log:  # never more than two requests hold a slot
        live += 1 if ev == "admit" else -1
        assert 0 <= live <= 2
    for rid, n in zip(rids, ns):
        (m, L), info = srv.result(rid)
        assert m.shape == (n + 1, 1) and L.shape == (n + 1, 1, 3)
        assert int(info["iterations"]) == 2 + n // 100
        assert info["calibrated"] is True
        assert srv.t_done[rid] >= srv.t_submit[rid]


def test_results_are_projected_per_request(fake):
    """result() applies the request's own E0 P: mean[:, 0] * p0, p0 the
    Nordsieck scale of its step."""
    srv = serve.Server(max_requests=4, max_points=10**6)
    ns = [100, 333]
    rids = [srv.submit(*logistic(n), order=2) for n in ns]
    _run(srv)
    for rid, n in zip(rids, ns):
        (m, _), _ = srv.result(rid)
        p0 = float(pbatch.prepare_rows([logistic(n)], 2)["p0"][0])
        assert torch.allclose(m[:, 0], torch.full((n + 1,), n * p0, dtype=torch.float64))


def test_memory_budget_keeps_fifo_within_a_shape(fake):
    """A request that does not fit waits, and later requests of the same
    shape wait behind it even if they would fit; other shapes go ahead."""
    srv = serve.Server(max_requests=8, max_points=1000)
    a = srv.submit(*logistic(600), order=2)
    b = srv.submit(*logistic(700), order=2)   # does not fit next to a
    c = srv.submit(*logistic(10), order=2)    # would fit, but b is first in line
    v = srv.submit(*vdp(500), order=3)        # another engine: admitted at once
    srv.tick()
    admitted = [(shape, n) for ev, shape, _, n in fake.log if ev == "admit"]
    assert admitted == [((3, 1), 600), ((8, 2), 500)]
    _run(srv)
    admitted = [n for ev, shape, _, n in fake.log if ev == "admit" and shape == (3, 1)]
    assert admitted == [600, 700, 10]
    for rid in (a, b, c, v):
        assert rid in srv.results
    assert not srv.busy()


def test_engines_per_shape_and_close(fake):
    srv = serve.Server(max_requests=4, max_points=10**5)
    srv.submit(*logistic(50), order=2)
    srv.submit(*logistic(50), order=3)
    srv.submit(*vdp(50), order=3)
    _run(srv)
    assert sorted(srv.engines) == [(1, 2), (1, 3), (2, 3)]
    srv.close()
    assert srv.engines == {}


def test_cancel_queued_and_running_requests(fake):
    """A queued request leaves the queue at once; an admitted one stops at
    the engine's next tick with its last iterate; both report "cancelled",
    and the other requests are unaffected."""
    srv = serve.Server(max_requests=1, max_points=10**6)
    a = srv.submit(*logistic(500), order=2)   # admitted, 7 iterations to go
    b = srv.submit(*logistic(100), order=2)   # waits for a's slot
    c = srv.submit(*logistic(200), order=2)
    srv.tick()
    assert srv.cancel(b)                      # still queued
    assert srv.cancel(a)                      # running
    _run(srv)
    (ma, _), ia = srv.result(a)
    assert ia["status"] == "cancelled" and int(ia["iterations"]) == 2  # one tick, then stopped at the next
    assert ma is not None and ma.shape == (501, 1)
    yb, ib = srv.result(b)
    assert yb is None and ib["status"] == "cancelled" and int(ib["iterations"]) == 0
    _, ic = srv.result(c)
    assert ic["status"] == "converged" and int(ic["iterations"]) == 2 + 200 // 100
    assert not srv.cancel(c)                  # already finished
    assert [n for ev, _, _, n in fake.log if ev == "admit"] == [500, 200]


def test_stuck_request_times_out(fake, monkeypatch):
    """A request that never meets its criterion (injected on the host: the
    fake engine never finishes it) is cancelled once its timeout has
    passed, reported as "timeout", and frees its slot for the next one."""
    clock = [0.0]
    monkeypatch.setattr(serve.time, "perf_counter", lambda: clock[0])
    fake.iterations = lambda n: 10**9 if n == 777 else 3
    srv = serve.Server(max_requests=1, max_points=10**6)
    stuck = srv.submit(*logistic(777), order=2, timeout=5.0)
    after = srv.submit(*logistic(50), order=2, timeout=5.0)
    for _ in range(4):
        srv.tick()
        clock[0] += 1.0
    assert stuck not in srv.results and after not in srv.results
    clock[0] = 5.0                            # both deadlines pass; `after` is still queued
    _run(srv)
    (m, _), info = srv.result(stuck)
    assert info["status"] == "timeout" and m.shape == (778, 1)
    y, info2 = srv.result(after)
    assert y is None and info2["status"] == "timeout"
    ev = [e for e, _, _, _ in fake.log]
    assert ev.count("cancel") == 1 and ev.count("admit") == 1


def test_mixed_precision_server(fake):
    """precision="mixed" creates mixed engines with the float32-phase
    settings and reports each request's float32 iterations (read before the
    result is fetched) beside the float64 ones."""
    srv = serve.Server(max_requests=4, max_points=10**6, precision="mixed", maxiters_f32=50, rtol_f32=1e-4,
                       settle_f32=0.1)
    rids = [srv.submit(*logistic(n), order=2) for n in (100, 222)]
    _run(srv)
    (h,) = list(fake.servers)
    assert fake.servers[h]["mixed"] == (50, 1e-4, 0.1)
    for rid, n in zip(rids, (100, 222)):
        _, info = srv.result(rid)
        assert int(info["iterations_float32"]) == n % 7 + 1
        assert int(info["iterations"]) == 2 + n // 100 and info["status"] == "converged"


# ---------------------------------------------------------------------------
# the dense lane (requests of pof._lib.DENSE_FIELDS, e.g. the reaction-diffusion
# system): libpof's host-driven solve replaced by a stand-in that "iterates"
# in its worker thread and checks the stop flag before every iteration
# ---------------------------------------------------------------------------

class FakeDenseSolve:
    def __init__(self, iterations):
        self.iterations = iterations  # n_steps -> iterations to convergence
        self.lock = threading.Lock()
        self.running = 0
        self.max_running = 0
        self.started = []

    def __call__(self, req, stop):
        with self.lock:
            self.running += 1
            self.max_running = max(self.max_running, self.running)
            self.started.append(req.rid)
        n = len(req.ts) - 1
        k, status = 0, 0
        while k < self.iterations(n):
            if stop():
                status = 3
                break
            time.sleep(0.002)
            k += 1
        with self.lock:
            self.running -= 1
        d = len(req.y0)
        D = d * (req.order + 1)
        ys = MVNSqrt(torch.full((n + 1, d), float(req.rid), dtype=torch.float64),
                     torch.zeros((n + 1, d, D), dtype=torch.float64))
        return ys, {"iterations": k, "nll": 1.0, "obj": 2.0, "sigma_squared": 3.0, "status": status}


def rd(n, cells=4):
    y0 = np.concatenate([-np.ones(cells), np.ones(cells)])
    return ("fhn_rd", (0.2, 0.2, 3.0, 0.5, 0.05), y0, np.linspace(0.0, 2.0, n + 1))


def _run_until_idle(srv, seconds=20.0):
    t0 = time.time()
    while srv.busy():
        srv.tick()
        time.sleep(0.001)
        assert time.time() - t0 < seconds
    return True


def test_dense_lane_overlaps_engines_and_keeps_its_budget(fake):
    """Dense-field requests run in the dense lane's worker threads while the
    engines serve the small-D requests; with a budget for one dense request
    at a time they start one after the other in arrival order; each gets its
    own result."""
    ds = FakeDenseSolve(iterations=lambda n: 5 + n // 50)
    probe = serve.Server(max_requests=4, max_points=10**6, dense_solve=ds)
    one = probe.dense.bytes_for(serve.Request(0, *rd(100), 3, 1e-6, 100))
    srv = serve.Server(max_requests=4, max_points=10**6, dense_solve=ds, dense_budget_bytes=one + 1)
    dr = [srv.submit(*rd(n), order=3) for n in (100, 60, 80)]
    sr = [srv.submit(*logistic(n), order=2) for n in (300, 120)]
    _run_until_idle(srv)
    assert ds.started == dr and ds.max_running == 1
    for rid, n in zip(dr, (100, 60, 80)):
        (m, L), info = srv.result(rid)
        assert m.shape == (n + 1, 8) and float(m[0, 0]) == rid
        assert info["status"] == "converged" and int(info["iterations"]) == 5 + n // 50
    for rid in sr:
        assert srv.result(rid)[1]["status"] == "converged"
    srv.close()


def test_dense_lane_runs_requests_side_by_side_within_budget(fake):
    ds = FakeDenseSolve(iterations=lambda n: 20)
    srv = serve.Server(max_requests=4, max_points=10**6, dense_solve=ds, dense_budget_bytes=1 << 40)
    rids = [srv.submit(*rd(50), order=2) for _ in range(3)]
    _run_until_idle(srv)
    assert ds.max_running >= 2
    assert all(srv.result(r)[1]["status"] == "converged" for r in rids)


def test_dense_lane_cancel_and_timeout(fake, monkeypatch):
    """A running dense request stops before its next iteration once
    cancelled (its last iterate returned, status "cancelled"), a queued one
    leaves the queue, and one past its deadline reports "timeout"."""
    ds = FakeDenseSolve(iterations=lambda n: 10**6 if n == 777 else 3)
    probe = serve.Server(max_requests=4, max_points=10**6, dense_solve=ds)
    one = probe.dense.bytes_for(serve.Request(0, *rd(777), 3, 1e-6, 100))
    srv = serve.Server(max_requests=4, max_points=10**6, dense_solve=ds, dense_budget_bytes=one + 1)
    a = srv.submit(*rd(777), order=3)           # runs "forever"
    b = srv.submit(*rd(20), order=3)            # waits behind a
    srv.tick()
    time.sleep(0.02)
    assert srv.cancel(b) and srv.cancel(a)
    _run_until_idle(srv)
    (ma, _), ia = srv.result(a)
    assert ia["status"] == "cancelled" and ma.shape == (778, 8)
    yb, ib = srv.result(b)
    assert yb is None and ib["status"] == "cancelled"
    c = srv.submit(*rd(777), order=3, timeout=0.05)
    _run_until_idle(srv)
    assert srv.result(c)[1]["status"] == "timeout"
    srv.close()


def test_taylor_mode_initial_values_in_two_threads():
    """The server's admission (pof.batch.prepare_rows) and a dense-lane worker
    (pof.solver.solve -> taylor_mode_init) compute Taylor-mode initial values
    with torch.func.jvp in different host threads; forward AD keeps its dual
    level in a process-wide counter, so both hold pof.utils.FORWARD_AD_LOCK.
    Run both side by side many times: no "no level exists" error."""
    from pof import initialization, ivp as pivp

    rd = pivp.fhn_reaction_diffusion(cells=4)
    errors = []

    def worker():
        try:
            for _ in range(40):
                initialization.taylor_mode_init(rd.f, rd.y0, 3, device=CPU)
        except Exception as e:  # noqa: BLE001
            errors.append(e)

    th = threading.Thread(target=worker)
    th.start()
    try:
        for _ in range(40):
            pbatch.prepare_rows([logistic(50)], 3)
            pbatch.prepare_rows([vdp(40)], 3)
    finally:
        th.join()
    assert not errors, errors[0]
