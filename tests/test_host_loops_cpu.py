"""The Python control loops of the drop-in package on CPU, with the one
device call they make -- libpof's filter/smoother -- replaced by the
oracle's.

`pof.solver.solve` for a user vector field (the loop of pof/solver.py:24-57
in Python: EK1 by torch.func, filter/smoother in libpof, crit read back each
iteration), `pof.iterators.ieks_iterator`, the quadratic-penalty iterator
(its regularization and tolerance schedule) and the Levenberg-Marquardt
iterator are compared iteration by iteration with the oracle's
restatements of the reference (oracle/solver.py).  What the substitution
leaves out -- libpof's own filter/smoother -- is what the GPU tests check.
"""

import sys

import numpy as np
import pytest
import torch

import pof.convenience  # noqa: F401  (every module that reads default_device is patched below)
import pof.initialization  # noqa: F401
import pof.observations  # noqa: F401
import pof.transitions  # noqa: F401
from oracle import filtsmooth as ofs, ivp as oivp, solver as osolver
from pof import iterators as pit, solver as psolver, step as pstep
from pof.utils import MVNSqrt

CPU = torch.device("cpu")


def _np(x):
    return np.ascontiguousarray(x.detach().cpu().numpy())


def oracle_filtsmooth(x0, dtm, dom):
    """pof.parallel_filtsmooth.linear_filtsmooth's contract, computed by the
    oracle on CPU tensors."""
    (m, L), nll, obj, ssq = ofs.linear_filtsmooth((_np(x0.mean), _np(x0.chol)), (_np(dtm.F), _np(dtm.QL)),
                                                  tuple(_np(a) for a in dom))

    def T(a):
        return torch.as_tensor(np.array(a, dtype=np.float64, copy=True), dtype=torch.float64)

    return MVNSqrt(T(m), T(L)), T(nll), T(obj), T(ssq)


@pytest.fixture
def host_only(monkeypatch):
    for name, mod in list(sys.modules.items()):
        if mod is not None and (name == "pof" or name.startswith("pof.")) and hasattr(mod, "default_device"):
            monkeypatch.setattr(mod, "default_device", lambda: CPU)
    monkeypatch.setattr(pstep, "parallel_linear_filtsmooth", oracle_filtsmooth)
    monkeypatch.setattr(pit, "fs", oracle_filtsmooth)


def user_field(name):
    """The same vector field as a plain torch function (no built-in tag: the
    package linearizes it with torch.func and loops in Python)."""
    if name == "logistic":
        return lambda t, y: 3.0 * y * (1.0 - y), [0.01], oivp.logistic(r=3.0), 10.0
    if name == "vanderpol":
        return (lambda t, y: torch.stack([y[1], 1.0 * ((1.0 - y[0] ** 2) * y[1] - y[0])]), [2.0, 0.0],
                oivp.vanderpol(stiffness_constant=1.0), 6.3)
    raise KeyError(name)


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("name,q,N,init", [("logistic", 2, 60, "constant"), ("logistic", 3, 120, "prior"),
                                           ("vanderpol", 3, 80, "constant")])
def test_solve_loop_for_a_user_field(host_only, name, q, N, init):
    f, y0, o, t1 = user_field(name)
    ts = np.linspace(0.0, t1, N)
    ys, info = psolver.solve(f=f, y0=y0, ts=ts, order=q, init=init)
    (om, oL), oinfo = osolver.solve(o, ts, q, init=init)
    assert int(info["iterations"]) == oinfo["iterations"]
    assert rel(_np(ys.mean), om) <= 1e-10
    C, oC = _np(ys.chol @ ys.chol.transpose(-1, -2)), oL @ np.swapaxes(oL, -1, -2)
    assert rel(C, oC) <= 1e-9
    for k in ("nll", "obj", "sigma_squared"):
        assert np.isclose(float(info[k]), oinfo[k], rtol=1e-9), k
    assert info["calibrated"] is True


def test_ieks_iterator_yields_the_same_iterations(host_only):
    f, y0, o, t1 = user_field("vanderpol")
    ts = np.linspace(0.0, t1, 70)
    it, _ = pit.ieks_iterator(f=f, y0=y0, ts=ts, order=2, init="constant")
    got = [(_np(s.mean), float(nll), float(obj)) for s, nll, obj, _ in it]
    oit, _ = osolver.ieks_iterator(o, ts, 2, init="constant")
    want = [(s[0], nll, obj) for s, nll, obj, _ in oit]
    assert len(got) == len(want) > 2
    for (m, nll, obj), (om, onll, oobj) in zip(got, want):
        assert rel(m, om) <= 1e-10 and np.isclose(nll, onll, rtol=1e-9) and np.isclose(obj, oobj, rtol=1e-9)


def test_quadratic_penalty_iterator_follows_the_schedule(host_only):
    """reg from 1e20 down by a factor per converged stage, snapped to 0
    below 1e-20, loop end once crit holds at reg = 0: the same regs, the same
    number of iterations and the same iterates as the oracle."""
    f, y0, o, t1 = user_field("logistic")
    ts = np.linspace(0.0, t1, 60)
    it, _ = pit.qpm_ieks_iterator(f=f, y0=y0, ts=ts, order=2, init="constant")
    got = [(_np(s.mean), float(obj), reg) for s, _, obj, reg in it]
    oit, setup = osolver.qpm_ieks_iterator(o, ts, 2, init="constant")
    want = [(s[0], obj, reg) for s, _, obj, reg in oit]
    assert len(got) == len(want) >= 42
    assert [r for _, _, r in got] == [r for _, _, r in want]
    assert want[-1][2] == 0.0
    for (m, obj, _), (om, oobj, _) in zip(got, want):
        assert rel(m, om) <= 1e-8 and np.isclose(obj, oobj, rtol=1e-8)


def test_levenberg_marquardt_iterator(host_only):
    """The regularized observation (d + D rows) runs through the same
    filter/smoother contract; the first iterations agree with the oracle."""
    f, y0, o, t1 = user_field("logistic")
    ts = np.linspace(0.0, t1, 40)
    setup = pof.convenience.set_up_solver(f=f, y0=y0, ts=ts, order=2)
    states = pof.convenience.get_initial_trajectory(setup, "constant")
    it = pit.lm_ieks_iterator(setup["dtm"], setup["om"], setup["x0"], MVNSqrt(states.mean[1:], states.chol[1:]),
                              reg=1.0)
    ost = osolver.set_up_solver(o, ts, 2)
    om0, _ = osolver.get_initial_trajectory(ost, "constant")
    oit = osolver.lm_ieks_iterator(ost, om0[1:], reg=1.0)
    for k in range(6):
        s, nll, obj, reg = next(it)
        os_, onll, oobj, oreg = next(oit)
        assert reg == oreg == 1.0
        assert rel(_np(s.mean), os_[0]) <= 1e-9
        assert np.isclose(float(nll), onll, rtol=1e-9) and np.isclose(float(obj), oobj, rtol=1e-9)


def _oracle_loop(st, init="constant", maxiters=10_000):
    """The reference's IEKS loop (solver.py:24-57) over any oracle set-up."""
    states = osolver.get_initial_trajectory(st, init)
    nll = obj = 0.0
    old, nll_old, obj_old = states, 0.0, 0.0
    k = 0
    while k < 1 or (not osolver.crit(obj, obj_old, nll, nll_old, states[0], old[0]) and k <= maxiters):
        old, nll_old, obj_old = states, nll, obj
        states, nll, obj, _ = osolver.ieks_step(st, old)
        k += 1
    return states, k


def test_non_uniform_grid_solve(host_only):
    """pof.solver.solve_nonuniform: per-step non-preconditioned transitions
    (the reference's set_up_solver_no_precond) on a grid refined towards
    t = 0.  Same iterations and means as the oracle's loop over the same
    set-up, and the solution of y' = y (1 - y), y(0) = 0.01, to 1e-6, where
    the reference's solve, taking every step as ts[1] - ts[0], is far off."""
    f = lambda t, y: y * (1.0 - y)  # noqa: E731
    o = oivp.logistic(r=1.0)
    u = np.linspace(0.0, 1.0, 50)
    ts = 10.0 * (1.0 - (1.0 - u) ** 2)
    exact = 1.0 / (1.0 + 99.0 * np.exp(-ts))
    ys, info = psolver.solve_nonuniform(f=f, y0=[0.01], ts=ts, order=3)
    st = osolver.set_up_solver_no_precond(o, ts, 3)
    (om, _), k = _oracle_loop(st)
    assert int(info["iterations"]) == k
    assert rel(_np(ys.mean), om @ st.E0.T) <= 1e-10
    assert np.abs(_np(ys.mean)[:, 0] - exact).max() < 1e-6
    (wrong, _), _ = osolver.solve(o, ts, 3, init="constant")
    assert np.abs(wrong[:, 0] - exact).max() > 1e-2


def test_non_preconditioned_set_up_on_a_uniform_grid(host_only):
    """On a uniform grid the Nordsieck preconditioning is only a change of
    coordinates: the same IEKS iterations and the same solution."""
    f = lambda t, y: y * (1.0 - y)  # noqa: E731
    ts = np.linspace(0.0, 10.0, 80)
    a, ia = psolver.solve(f=f, y0=[0.01], ts=ts, order=3, init="constant")
    b, ib = psolver.solve_nonuniform(f=f, y0=[0.01], ts=ts, order=3)
    assert int(ia["iterations"]) == int(ib["iterations"])
    assert rel(_np(b.mean), _np(a.mean)) <= 1e-11


def test_loops_stop_on_nan(host_only, monkeypatch):
    """The reference stops on NaN (convergence_criteria.py:6,
    iterators.py:105-106): a filter/smoother that returns a NaN objective on
    its second call ends the solve loop and the QPM loop there, and the NaN
    reaches info."""
    calls = []

    def poisoned(x0, dtm, dom):
        calls.append(1)
        out, nll, obj, ssq = oracle_filtsmooth(x0, dtm, dom)
        if len(calls) >= 2:
            obj = torch.tensor(float("nan"), dtype=torch.float64)
        return out, nll, obj, ssq

    monkeypatch.setattr(pstep, "parallel_linear_filtsmooth", poisoned)
    monkeypatch.setattr(pit, "fs", poisoned)
    f, y0, _, t1 = user_field("vanderpol")
    ts = np.linspace(0.0, t1, 50)
    _, info = psolver.solve(f=f, y0=y0, ts=ts, order=2, init="constant")
    assert int(info["iterations"]) == 2 and torch.isnan(info["obj"])
    calls.clear()
    it, _ = pit.qpm_ieks_iterator(f=f, y0=y0, ts=ts, order=2, init="constant")
    assert len(list(it)) == 2


def test_sequential_eks_of_a_user_field(host_only, monkeypatch):
    """pof.solver.sequential_eks_solve for a plain torch field: the EKF
    step by step in torch (filter.py:9-30, linearized at each predicted mean)
    and the RTS smoother (here the oracle's in place of libpof's) give the
    oracle's sequential EKS (solver.py:76-96)."""
    import pof.parallel_filtsmooth as ppfs

    def oracle_smoothing(dtm, filt):
        (m, L), obj = ofs.sequential_smoothing((_np(dtm[0]), _np(dtm[1])), (_np(filt[0]), _np(filt[1])))
        return MVNSqrt(torch.as_tensor(m.copy()), torch.as_tensor(L.copy())), torch.tensor(obj)

    monkeypatch.setattr(ppfs, "smoothing", oracle_smoothing)
    f, y0, o, t1 = user_field("vanderpol")
    ts = np.linspace(0.0, t1, 60)
    ys, info = psolver.sequential_eks_solve(f=f, y0=y0, ts=ts, order=3)
    (om, oL), oinfo = osolver.sequential_eks_solve(o, ts, 3)
    assert rel(_np(ys.mean), om) <= 1e-10
    C, oC = _np(ys.chol @ ys.chol.transpose(-1, -2)), oL @ np.swapaxes(oL, -1, -2)
    assert rel(C, oC) <= 1e-9
    for k in ("nll", "obj", "sigma_squared"):
        assert np.isclose(float(info[k]), oinfo[k], rtol=1e-9), k
    full, _ = psolver.sequential_eks_solve(f=f, y0=y0, ts=ts, order=3, return_full_states=True)
    (ofull, _), _ = osolver.sequential_eks_solve(o, ts, 3, return_full_states=True)
    assert rel(_np(full.mean), ofull) <= 1e-10


# ---------------------------------------------------------------------------
# the host-driven float32 phase of precision="mixed" (pof.solver._float32_phase,
# the rules of pof_ieks_solve_mixed): its stopping and discard rules against a
# scripted sequence of float32 iterates (libpof's linearization and
# filter/smoother replaced by fakes that move y = E0 m by chosen amounts)
# ---------------------------------------------------------------------------

def _phase_setup(monkeypatch, rels):
    from pof.observations import AffineModel
    from pof.transitions import TransitionModel

    n, D = 6, 2
    E0 = torch.tensor([[1.0, 0.0]], dtype=torch.float64)
    F = torch.eye(D, dtype=torch.float64).expand(n, D, D)
    setup = {"dtm": TransitionModel(F, F), "om": object(), "E0": E0,
             "x0": MVNSqrt(torch.zeros(D, dtype=torch.float64), torch.zeros((D, D), dtype=torch.float64))}
    states = MVNSqrt(torch.ones((n + 1, D), dtype=torch.float64), torch.zeros((n + 1, D, D), dtype=torch.float64))
    cur = {"m": states.mean.clone(), "calls": 0}
    script = iter(rels)

    def lin(om, st):
        return AffineModel(torch.ones((n, 1, D), dtype=torch.float64), torch.zeros((n, 1), dtype=torch.float64), None)

    def fs(x0, dtm, dom):
        cur["calls"] += 1
        assert dtm[0].dtype == torch.float32 and dom[0].dtype == torch.float32 and dtm[0].dim() == 2
        r = next(script)
        m = cur["m"].clone()
        m[:, 0] = m[:, 0] * (1.0 + r) if np.isfinite(r) else float("nan")
        if np.isfinite(r):
            cur["m"] = m
        return MVNSqrt(m.to(torch.float32), None), None, None, None

    monkeypatch.setattr(pstep, "linearize_at_previous_states", lin)
    monkeypatch.setattr(psolver, "parallel_linear_filtsmooth", fs)
    monkeypatch.setattr(psolver, "_wait", lambda dev: None)
    return setup, states, cur


@pytest.mark.parametrize("rels,kw,expect_it,expect_kept", [
    # converges: the change falls below rtol_f32 at the 5th iteration
    ([0.5, 0.1, 0.01, 1e-3, 1e-6], dict(rtol_f32=1e-5), 5, True),
    # three changes that do not shrink (settle_f32 = inf counts from the first): stops, and
    # the phase never came within 100 rtol_f32 -> discarded
    ([0.5, 0.6, 0.7, 0.8, 0.9], dict(rtol_f32=1e-5), 4, False),
    # a non-finite float32 iterate ends the phase; the one kept iteration is within 100 rtol_f32
    ([0.1, float("nan")], dict(rtol_f32=0.01), 1, True),
    # non-shrinking changes count only once the smallest change is below settle_f32
    ([0.5, 0.7, 0.9, 0.01, 0.02, 0.03, 0.04, 0.05], dict(rtol_f32=1e-3, settle_f32=0.05), 7, True),
    # maxiters_f32
    ([0.5, 0.4, 0.3, 0.2, 0.1], dict(rtol_f32=1e-3, maxiters_f32=3), 3, False),
])
def test_float32_phase_rules(monkeypatch, rels, kw, expect_it, expect_kept):
    setup, states, cur = _phase_setup(monkeypatch, rels)
    args = dict(maxiters_f32=100, rtol_f32=1e-5, settle_f32=float("inf"))
    args.update(kw)
    means, it32, best = psolver._float32_phase(setup, states, **args)
    if expect_kept:
        assert it32 == expect_it
        assert torch.allclose(means, cur["m"], rtol=1e-6)  # the last finite float32 iterate, in float64
    else:
        assert it32 == 0 and torch.equal(means, states.mean)  # discarded: the input trajectory
    finite = [r for r in rels[:expect_it] if np.isfinite(r)]
    assert best == pytest.approx(min(finite), rel=1e-3, abs=1e-7)  # measured on float32 iterates


def test_float32_phase_stop_hook(monkeypatch):
    setup, states, cur = _phase_setup(monkeypatch, [0.5, 0.4, 0.3, 0.2, 0.1])
    calls = {"n": 0}

    def stop():
        calls["n"] += 1
        return calls["n"] > 2  # two iterations, then stop

    means, it32, best = psolver._float32_phase(setup, states, 100, 1e-5, float("inf"), stop)
    assert cur["calls"] == 2


def test_solve_loop_stop_hook_and_status(host_only):
    """solve(..., stop=...) for a field without a device loop: the hook is
    checked before every iteration; once it returns True the loop ends with
    the last iterate and status 3 (cancelled).  rtol reaches crit."""
    f, y0, _, t1 = user_field("vanderpol")
    ts = np.linspace(0.0, t1, 40)
    (m_full, _), full = psolver.solve(f=f, y0=y0, ts=ts, order=2, init="constant")
    assert int(full["status"]) == 0 and int(full["iterations"]) > 3
    calls = {"n": 0}

    def stop_after(k):
        def stop():
            calls["n"] += 1
            return calls["n"] > k
        return stop

    _, info0 = psolver.solve(f=f, y0=y0, ts=ts, order=2, init="constant", stop=stop_after(0))
    assert int(info0["status"]) == 3 and int(info0["iterations"]) == 0
    calls["n"] = 0
    _, info2 = psolver.solve(f=f, y0=y0, ts=ts, order=2, init="constant", stop=stop_after(2))
    assert int(info2["status"]) == 3 and int(info2["iterations"]) == 2
    # a looser objective tolerance stops no later
    _, loose = psolver.solve(f=f, y0=y0, ts=ts, order=2, init="constant", rtol=1e-2)
    assert int(loose["status"]) == 0 and int(loose["iterations"]) <= int(full["iterations"])
