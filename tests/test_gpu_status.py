"""Failure detection on the GPU without a GPU fault: every stop of an IEKS
loop carries a status word (info[POF_I_STATUS]: converged, maxiters,
nonfinite, cancelled).  Poisoned inputs -- NaN in y0 or in a field's
parameters -- are safe to run: NaN propagates through the arithmetic and the
reference's criterion stops the loop on it (pof/convergence_criteria.py:6),
nothing traps.  A poisoned problem of a batch does not touch the others
(bit-identical to the batch without it), and a served request cancelled by
its host flag stops at the next tick."""

import numpy as np
import pytest
import torch

from pof import _lib, batch as pbatch, ivp as pivp, serve, solver as psolver

pytestmark = pytest.mark.gpu


def test_solve_status_converged_and_maxiters():
    p = pivp.vanderpol(stiffness_constant=1.0)
    ts = np.linspace(0.0, 6.3, 128)
    _, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=3, init="constant")
    assert _lib.solve_status(int(info["status"])) == "converged"
    _, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=3, init="constant", maxiters=2)
    assert int(info["iterations"]) == 3  # the reference's loop allows maxiters + 1 (solver.py:41)
    assert _lib.solve_status(int(info["status"])) == "maxiters"
    _, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=3, init="constant", sequential=True, maxiters=1)
    assert _lib.solve_status(int(info["status"])) == "maxiters"


@pytest.mark.parametrize("sequential", [False, True])
def test_nan_initial_value_stops_after_the_first_iteration(sequential):
    """y0 = (NaN, 0): the first iteration always runs (solver.py:24-45) and
    yields a NaN objective; crit stops the loop on it, the status says why,
    as the reference's loop does (its first cond check after iteration 1 sees
    the NaN)."""
    p = pivp.vanderpol(stiffness_constant=1.0)
    ts = np.linspace(0.0, 6.3, 64)
    ys, info = psolver.solve(f=p.f, y0=[float("nan"), 0.0], ts=ts, order=3, init="constant", sequential=sequential)
    assert int(info["iterations"]) == 1
    assert _lib.solve_status(int(info["status"])) == "nonfinite"
    assert torch.isnan(info["obj"]) or torch.isnan(info["nll"])


def _batch(spec, q, maxiters=1000):
    problems = [(nm, p, y0, np.linspace(0.0, t1, N)) for (nm, p, y0, t1, N) in spec]
    return pbatch.solve_batch(problems, order=q, maxiters=maxiters)


def test_poisoned_problem_of_a_batch_leaves_the_others_alone():
    """A NaN parameter in one problem of a batch: that problem stops after
    its first iteration with status "nonfinite"; every other problem's
    result and info are bit-identical to the batch without it."""
    good = [("vanderpol", (1.0,), [2.0, 0.0], 6.3, 128), ("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], 7.0, 150),
            ("vanderpol", (1.2,), [1.9, 0.1], 5.0, 257)]
    bad = ("vanderpol", (float("nan"),), [2.0, 0.0], 6.3, 200)
    a = _batch(good, 3)
    b = _batch(good[:1] + [bad] + good[1:], 3)
    (_, _), ib = b.problem(1)
    assert int(ib["iterations"]) == 1 and _lib.solve_status(int(ib["status"])) == "nonfinite"
    for i, j in ((0, 0), (1, 2), (2, 3)):
        (ma, La), ia = a.problem(i)
        (mb, Lb), ibb = b.problem(j)
        assert torch.equal(ma, mb) and torch.equal(La, Lb)
        for k in ("iterations", "obj", "nll", "sigma_squared", "status"):
            assert float(ia[k]) == float(ibb[k]), k
        if i != 1:  # the Van der Pol problems converge (Lotka-Volterra may run to maxiters)
            assert _lib.solve_status(int(ia["status"])) == "converged"


def test_batch_status_maxiters():
    r = _batch([("vanderpol", (1.0,), [2.0, 0.0], 6.3, 128)], 3, maxiters=1)
    (_, _), info = r.problem(0)
    assert int(info["iterations"]) == 2 and _lib.solve_status(int(info["status"])) == "maxiters"


def test_cancelled_request_stops_and_the_others_are_unaffected():
    """pof_server_cancel sets a host flag that the engine reads at each tick:
    the cancelled request finishes at the next tick with status
    "cancelled" and fewer iterations than it needs; the request beside it
    gets the result it gets alone."""
    reqs = [("vanderpol", (1.0,), [2.0, 0.0], np.linspace(0.0, 6.3, 300), 3),
            ("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], np.linspace(0.0, 7.0, 400), 3)]

    def run(cancel):
        srv = serve.Server(max_requests=8, max_points=1 << 14)
        rids = [srv.submit(nm, p, y0, ts, q, maxiters=1000) for (nm, p, y0, ts, q) in reqs]
        srv.tick()
        srv.tick()
        if cancel:
            assert srv.cancel(rids[0])
        guard = 0
        while srv.busy():
            srv.tick()
            guard += 1
            assert guard < 5000
        out = [srv.result(r) for r in rids]
        srv.close()
        return out

    alone = run(False)
    cut = run(True)
    assert alone[0][1]["status"] == "converged"
    assert cut[0][1]["status"] == "cancelled"
    assert int(cut[0][1]["iterations"]) == 3 < int(alone[0][1]["iterations"])
    (ma, La), ia = alone[1]
    (mb, Lb), ib = cut[1]
    assert torch.equal(ma, mb) and torch.equal(La, Lb) and ib["status"] == ia["status"] == "converged"
