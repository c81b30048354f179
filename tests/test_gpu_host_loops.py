"""The drop-in package's Python loops with libpof doing the filter/smoother
on the GPU (the CPU tests of the same loops put the oracle in libpof's
place): the quadratic-penalty IEKS iterator (pof/iterators.py:53-106), the
Levenberg-Marquardt-regularized iterator, whose observation model has
d + D rows (pof/iterators.py:109-133, pof/observations.py:64-83), and the
non-uniform-grid solve over the reference's non-preconditioned per-step
set-up (pof/convenience.py:48-73), each against the oracle's restatement;
plus the (D, d) = (12, 2) and (12, 3) shapes of the scan-length sweep's
q = 5 and of the rigid body at q = 3, parallel and sequential."""

import numpy as np
import pytest
import torch

import pof.convenience
from oracle import ivp as oivp, solver as osolver
from oracle.scan import sequential_scan
from pof import _lib, ivp as pivp, iterators as pit, solver as psolver
from pof.utils import MVNSqrt

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _np(x):
    return np.ascontiguousarray(x.detach().cpu().numpy())


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def logistic_field(t, y):
    return 3.0 * y * (1.0 - y)


def test_quadratic_penalty_iterator_on_the_gpu():
    """reg from 1e20 down by a factor per converged stage, 0 below 1e-20, the
    loop's end once crit holds at reg = 0: the same regs, the same number of
    iterations and (within 1e-8) the same iterates as the oracle, with the
    filter/smoother (R = reg I / N, a noise model the EK1 loop never has) in
    libpof."""
    ts = np.linspace(0.0, 10.0, 60)
    it, _ = pit.qpm_ieks_iterator(f=logistic_field, y0=[0.01], ts=ts, order=2, init="constant")
    got = [(_np(s.mean), float(obj), reg) for s, _, obj, reg in it]
    oit, _ = osolver.qpm_ieks_iterator(oivp.logistic(r=3.0), ts, 2, init="constant")
    want = [(s[0], obj, reg) for s, _, obj, reg in oit]
    assert len(got) == len(want) >= 42
    assert [r for _, _, r in got] == [r for _, _, r in want]
    worst = max(rel(m, om) for (m, _, _), (om, _, _) in zip(got, want))
    print("[qpm] %d iterations, largest mean difference %.3g" % (len(got), worst))
    assert worst <= 1e-8
    for (_, obj, _), (_, oobj, _) in zip(got, want):
        assert np.isclose(obj, oobj, rtol=1e-8)


def test_levenberg_marquardt_iterator_on_the_gpu():
    """The regularized model stacks the EK1 row over the D rows of I with
    noise blockdiag(0, I / sqrt(reg)): (D, d + D) = (3, 4), a shape with more
    observation rows than states, through libpof's filter/smoother.  Its
    first eight iterations equal the oracle's."""
    assert _lib.shape_supported(3, 4)
    ts = np.linspace(0.0, 10.0, 40)
    setup = pof.convenience.set_up_solver(f=logistic_field, y0=[0.01], ts=ts, order=2)
    states = pof.convenience.get_initial_trajectory(setup, "constant")
    it = pit.lm_ieks_iterator(setup["dtm"], setup["om"], setup["x0"], MVNSqrt(states.mean[1:], states.chol[1:]),
                              reg=1.0)
    ost = osolver.set_up_solver(oivp.logistic(r=3.0), ts, 2)
    om0, _ = osolver.get_initial_trajectory(ost, "constant")
    oit = osolver.lm_ieks_iterator(ost, om0[1:], reg=1.0)
    # the first eight iterations (the loop ends only when nll and obj both
    # stall, which on this problem takes thousands of iterations)
    got = [(_np(s.mean), float(nll), float(obj), reg) for (s, nll, obj, reg), _ in zip(it, range(8))]
    want = [(s[0], nll, obj, reg) for (s, nll, obj, reg), _ in zip(oit, range(8))]
    assert len(got) == len(want) == 8
    for (m, nll, obj, reg), (om, onll, oobj, oreg) in zip(got, want):
        assert reg == oreg == 1.0
        assert rel(m, om) <= 1e-9
        assert np.isclose(nll, onll, rtol=1e-9) and np.isclose(obj, oobj, rtol=1e-9)


def _oracle_loop(st, init="constant", maxiters=10_000, scan=None):
    states = osolver.get_initial_trajectory(st, init)
    nll = obj = 0.0
    old, nll_old, obj_old = states, 0.0, 0.0
    k = 0
    kw = {} if scan is None else {"scan": scan}
    while k < 1 or (not osolver.crit(obj, obj_old, nll, nll_old, states[0], old[0]) and k <= maxiters):
        old, nll_old, obj_old = states, nll, obj
        states, nll, obj, _ = osolver.ieks_step(st, old, **kw)
        k += 1
    return states, k


def test_non_uniform_grid_solve_on_the_gpu():
    """pof.solver.solve_nonuniform: one non-preconditioned transition per
    step (per-step F, Q_L stacks into libpof) on a grid refined towards
    t = 0: the oracle's iterations and means, and the exact solution of
    y' = y (1 - y), y(0) = 0.01, to 1e-6."""
    f = lambda t, y: y * (1.0 - y)  # noqa: E731
    u = np.linspace(0.0, 1.0, 50)
    ts = 10.0 * (1.0 - (1.0 - u) ** 2)
    exact = 1.0 / (1.0 + 99.0 * np.exp(-ts))
    ys, info = psolver.solve_nonuniform(f=f, y0=[0.01], ts=ts, order=3)
    st = osolver.set_up_solver_no_precond(oivp.logistic(r=1.0), ts, 3)
    (om, _), k = _oracle_loop(st)
    (sm, _), ks = _oracle_loop(st, scan=sequential_scan)
    assert int(info["iterations"]) == k == ks
    # the two oracle orders differ by 1.6e-9 on this grid (steps from 0.4 down
    # to 4e-3): the fixed point amplifies rounding by its conditioning
    spread = rel(sm @ st.E0.T, om @ st.E0.T)
    tol = max(TOL, 10 * spread)
    print("[non-uniform] gpu vs oracle %.3g, tolerance %.3g (oracle order spread %.3g)" % (
        rel(_np(ys.mean), om @ st.E0.T), tol, spread))
    assert spread <= 5e-9
    assert rel(_np(ys.mean), om @ st.E0.T) <= tol
    assert np.abs(_np(ys.mean)[:, 0] - exact).max() < 1e-6


SHAPES_12 = [
    ("fhn_q5", lambda: (pivp.fhn_classic(tmax=10.0), oivp.fhn_classic(tmax=10.0)), 10.0, 120, 5),
    ("rigid_q3", lambda: (pivp.rigid_body(), oivp.rigid_body()), None, 100, 3),
]


@pytest.mark.parametrize("name,mk,t1,N,q", SHAPES_12)
@pytest.mark.parametrize("sequential", [False, True])
def test_d12_solves(name, mk, t1, N, q, sequential):
    """D = 12: FitzHugh-Nagumo at q = 5 (d = 2) and the rigid body at q = 3
    (d = 3), the whole IEKS loop in libpof (parallel scans, or the sequential
    filter/smoother: one chunk spanning the grid), against the oracle in the
    matching order: same iteration count, means within 1e-10 or 10x the
    spread of the oracle's two orders."""
    p, o = mk()
    assert _lib.shape_supported(12, o.y0.shape[0])
    t1 = o.tmax if t1 is None else t1
    ts = np.linspace(o.t0, t1, N)
    (om, _), oinfo = osolver.solve(o, ts, q, init="constant", maxiters=1000, sequential=sequential)
    (am, _), ainfo = osolver.solve(o, ts, q, init="constant", maxiters=1000,
                                   **({"scan": sequential_scan} if not sequential else {"sequential": False}))
    out, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=q, init="constant", maxiters=1000, sequential=sequential)
    tol = max(TOL, 10 * rel(am, om))
    print("[%s seq=%s] iterations gpu %d oracle %d/%d, tolerance %.3g" % (
        name, sequential, int(info["iterations"]), oinfo["iterations"], ainfo["iterations"], tol))
    assert tol <= 1e-8
    assert int(info["iterations"]) == oinfo["iterations"]
    assert rel(_np(out.mean), om) <= tol
    assert _lib.solve_status(int(info["status"])) == "converged"
