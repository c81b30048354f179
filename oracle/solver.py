"""Problem set-up, EK1 linearization, initial trajectories, convergence
criterion and the IEKS loop, restated in NumPy float64 (test infrastructure).

Restates ``pof/convenience.py`` (both set-ups), ``pof/initialization.py``,
``pof/observations.py``, ``pof/step.py``, ``pof/convergence_criteria.py``,
``pof/solver.py`` and the IEKS, quadratic-penalty and Levenberg-Marquardt
iterators of ``pof/iterators.py``, including the reference's quirks:

* double calibration of the returned chol (``step.py:42-44`` and
  ``solver.py:66-69``);
* ``prior`` init uses absolute times as step sizes, non-preconditioned
  transitions and is not multiplied by PI (``initialization.py:83-89``,
  ``convenience.py:88-90``);
* the first IEKS iteration always runs and compares against zeros
  (``solver.py:24-45``).
"""

from typing import NamedTuple

import numpy as np

from . import core, filtsmooth, taylor
from .scan import associative_scan


class Setup(NamedTuple):
    ivp: object
    ts: np.ndarray
    d: int
    q: int
    F: np.ndarray  # (N-1, D, D)
    QL: np.ndarray  # (N-1, D, D)
    P: np.ndarray
    PI: np.ndarray
    E0: np.ndarray  # E0 @ P
    E1: np.ndarray  # E1 @ P
    x0: tuple  # (m0, L0) preconditioned


def taylor_mode_init(ivp, q):
    """``initialization.py:15-22``: mean = derivatives (dimension-major), chol = 0."""
    derivs = taylor.taylor_derivatives(ivp.components, ivp.y0, q)  # (q+1, d)
    d = ivp.y0.shape[0]
    m0 = np.concatenate(derivs.T)
    P0 = np.kron(np.eye(d), np.zeros((q + 1, q + 1)))
    return m0, P0


def set_up_solver(ivp, ts, order):
    """``convenience.py:13-45``."""
    ts = np.asarray(ts, dtype=np.float64)
    dt = (ts[1:] - ts[:-1])[0]
    d = ivp.y0.shape[0]
    q = order
    A, QL = core.preconditioned_discretize(d, q)
    n = ts.shape[0] - 1
    F = np.broadcast_to(A, (n,) + A.shape).copy()
    QLs = np.broadcast_to(QL, (n,) + QL.shape).copy()
    P, PI = core.nordsieck_preconditioner(d, q, dt)
    E0 = core.projection_matrix(d, q, 0) @ P
    E1 = core.projection_matrix(d, q, 1) @ P
    m0, L0 = taylor_mode_init(ivp, q)
    x0 = (PI @ m0, PI @ L0)
    return Setup(ivp, ts, d, q, F, QLs, P, PI, E0, E1, x0)


def set_up_solver_no_precond(ivp, ts, order):
    """``convenience.py:48-73``: per-step NON-preconditioned transitions at
    the grid's own step sizes (so a non-uniform grid is honoured), P = PI =
    I, plain projections, x0 by Taylor mode."""
    ts = np.asarray(ts, dtype=np.float64)
    d = ivp.y0.shape[0]
    q = order
    F, QL = core.discretize_transitions(d, q, ts[1:] - ts[:-1])
    D = d * (q + 1)
    I = np.eye(D)
    E0 = core.projection_matrix(d, q, 0)
    E1 = core.projection_matrix(d, q, 1)
    return Setup(ivp, ts, d, q, F, QL, I, I, E0, E1, taylor_mode_init(ivp, q))


def observation_residual(setup, x):
    """The ``NonlinearModel`` of ``convenience.py:28``: E1 x - f(E0 x)."""
    y = filtsmooth.mv(setup.E0, x)
    return filtsmooth.mv(setup.E1, x) - setup.ivp.f(None, y)


def linearize(setup, m):
    """``observations.py:35-40`` (EK1, jacfwd): H = d om / dx, c = om(m) - H m, cholR = 0."""
    y = filtsmooth.mv(setup.E0, m)
    J = setup.ivp.jac(y)  # (..., d, d)
    H = setup.E1 - J @ setup.E0
    res = filtsmooth.mv(setup.E1, m) - setup.ivp.f(None, y)
    c = res - filtsmooth.mv(H, m)
    d = setup.d
    R = np.zeros(m.shape[:-1] + (d, d))
    return H, c, R


def linearize_at_previous_states(setup, means):
    """``step.py:12-22``: linearize at states[1:]."""
    return linearize(setup, means[1:])


# --------------------------------------------------------------------------
# initial trajectories, initialization.py / convenience.py:76-92
# --------------------------------------------------------------------------


def constant_init(ivp, order, ts):
    """``initialization.py:42-56``."""
    y0 = ivp.y0
    d = y0.shape[-1]
    N = len(ts)
    dy0 = ivp.f(None, y0)
    x0 = np.concatenate([y0[:, None], dy0[:, None], np.zeros((d, order - 1))], axis=1)
    x0 = x0.reshape(1, -1)
    traj = np.repeat(x0, N, axis=0)
    D = traj.shape[1]
    return traj, np.zeros((N, D, D))


def prior_init(ivp, order, ts):
    """``initialization.py:75-89``: one-step predictions from x0 with the
    NON-preconditioned transitions at step sizes ``ts[1:]`` (absolute times)."""
    m0, L0 = taylor_mode_init(ivp, order)
    d = ivp.y0.shape[0]
    F, QL = core.discretize_transitions(d, order, np.asarray(ts)[1:])
    pm, pL = filtsmooth.sqrt_predict(F, QL, m0[None], L0[None])
    means = np.concatenate([m0[None], pm])
    chols = np.concatenate([L0[None], pL])
    return means, chols


def coarse_ekf_init(ivp, order, ts, N=10):
    """``initialization.py:112-129`` (a sequential EKS on a coarse grid, full states)."""
    ts = np.asarray(ts)
    coarse_ts = np.linspace(ts[0], ts[-1], N)
    coarse_dt = coarse_ts[1] - coarse_ts[0]
    (means, chols), _ = sequential_eks_solve(ivp, coarse_ts, order, return_full_states=True)
    idxs = np.floor(ts / coarse_dt).astype(int)
    return means[idxs], chols[idxs]


def get_initial_trajectory(setup, method="prior"):
    """``convenience.py:76-92``."""
    ivp, ts, q, PI = setup.ivp, setup.ts, setup.q, setup.PI
    if method == "coarse":
        m, L = coarse_ekf_init(ivp, q, ts, N=100)
        return m @ PI.T, PI @ L
    if method == "constant":
        m, L = constant_init(ivp, q, ts)
        return m @ PI.T, PI @ L
    if method == "prior":
        return prior_init(ivp, q, ts)
    raise Exception(f"method={method} not found")


# --------------------------------------------------------------------------
# loop
# --------------------------------------------------------------------------


def crit(obj, obj_old, nll, nll_old, means, means_old, *, rtol=1e-6, atol=1e-9):
    """``convergence_criteria.py:4-13`` (means test: rtol 1e-13, atol 1e-8 default)."""
    isnan = np.isnan(obj) or np.isnan(nll)
    obj_converged = bool(np.isclose(obj_old, obj, rtol=rtol, atol=atol))
    means_converged = bool(np.isclose(means_old, means, rtol=1e-13).all())
    return bool(isnan or obj_converged or means_converged)


def ieks_step(setup, states, calibrate=True, sequential=False, scan=associative_scan, filtsmooth_fn=None):
    """``step.py:33-45``.  filtsmooth_fn(x0, dtm, dom) replaces the parallel
    filter/smoother (another bracketing of the same scans)."""
    dtm = (setup.F, setup.QL)
    dom = linearize_at_previous_states(setup, states[0])
    if filtsmooth_fn is not None:
        out, nll, obj, ssq = filtsmooth_fn(setup.x0, dtm, dom)
    elif not sequential:
        out, nll, obj, ssq = filtsmooth.linear_filtsmooth(setup.x0, dtm, dom, scan=scan)
    else:
        out, nll, obj, ssq = filtsmooth.sequential_linear_filtsmooth(setup.x0, dtm, dom)
    if calibrate:
        out = (out[0], ssq**0.5 * out[1])
    return out, nll, obj, ssq


def solve(ivp, ts, order, init="prior", calibrate=True, maxiters=10_000, sequential=False,
          scan=associative_scan, return_full=False, callback=None, filtsmooth_fn=None, rtol=1e-6):
    """``solver.py:11-73``: returns ((means (N,d), chols (N,d,D)), info)."""
    setup = set_up_solver(ivp, ts, order)
    states = get_initial_trajectory(setup, method=init)
    nll = obj = ssq = 0.0
    states_old, nll_old, obj_old = states, 0.0, 0.0
    k = 0
    while True:
        # cond (solver.py:36-45)
        first = k < 1
        not_max = k <= maxiters
        conv = crit(obj, obj_old, nll, nll_old, states[0], states_old[0], rtol=rtol)
        if not (first or ((not conv) and not_max)):
            break
        # body (solver.py:47-55)
        states_old, nll_old, obj_old = states, nll, obj
        states, nll, obj, ssq = ieks_step(setup, states_old, sequential=sequential, scan=scan,
                                          filtsmooth_fn=filtsmooth_fn)
        k += 1
        if callback is not None:
            callback(k, states, nll, obj, ssq)
    info = {"iterations": k, "nll": nll, "obj": obj, "sigma_squared": ssq, "calibrated": False}
    if calibrate:
        states = (states[0], ssq**0.5 * states[1])
        info["calibrated"] = True
    if return_full:
        return states, info, setup
    ys = (states[0] @ setup.E0.T, setup.E0 @ states[1])
    return ys, info


def sequential_eks_solve(ivp, ts, order, return_full_states=False, calibrate=True):
    """``solver.py:76-96``: one EKF + RTS pass, linearizing at predicted means."""
    setup = set_up_solver(ivp, ts, order)
    dtm = (setup.F, setup.QL)

    def lin(m):
        H, c, R = linearize(setup, m[None])
        return H[0], c[0], R[0]

    states, nll, obj, ssq = filtsmooth.sequential_filtsmooth(setup.x0, dtm, lin)
    info = {"nll": nll, "obj": obj, "sigma_squared": ssq, "calibrated": False}
    if calibrate:
        states = (states[0], ssq**0.5 * states[1])
        info["calibrated"] = True
    M = setup.P if return_full_states else setup.E0
    return (states[0] @ M.T, M @ states[1]), info


def ieks_iterator(ivp, ts, order, init="prior"):
    """``iterators.py:20-41``: yields (states, nll, obj, ssq) until ``crit``."""
    setup = set_up_solver(ivp, ts, order)
    states = get_initial_trajectory(setup, method=init)

    def gen():
        st, nll, obj, ssq = ieks_step(setup, states)
        yield st, nll, obj, ssq
        while True:
            nll_old, obj_old, st_old = nll, obj, st
            st, nll, obj, ssq = ieks_step(setup, st_old)
            yield st, nll, obj, ssq
            if crit(obj, obj_old, nll, nll_old, st[0], st_old[0]):
                break

    return gen(), setup


# --------------------------------------------------------------------------
# regularized IEKS iterators, iterators.py:44-133
# --------------------------------------------------------------------------


def qpm_ieks_iterator(ivp, ts, order, init="prior", reg_start=1e20, reg_final=1e-20, steps=40, tau_start=None,
                      tau_final=None):
    """``iterators.py:44-106``, quadratic-penalty IEKS: the EK1 model with
    noise chol ``reg * I / N`` (N = number of steps); each time ``crit``
    holds at tolerance tau, reg and tau shrink geometrically, reg snaps to 0
    below reg_final and the loop ends once crit holds at reg = 0 (or on NaN).
    No calibration (the filter/smoother is called directly).  Yields
    (states, nll, obj, reg).  The reference's ``init_covs`` lines compute a
    value nothing reads and are left out."""
    setup = set_up_solver(ivp, ts, order)
    states = get_initial_trajectory(setup, method=init)
    dtm = (setup.F, setup.QL)
    N = setup.F.shape[0]
    if tau_start is None:
        tau_start, tau_final = 1e5, 1e-5
    reg_fact = (reg_final / reg_start) ** (1 / steps)
    tau_fact = (tau_final / tau_start) ** (1 / steps)

    def gen():
        reg, tau = reg_start, tau_start
        H, c, R = linearize_at_previous_states(setup, states[0])
        eye = np.broadcast_to(np.eye(R.shape[-1]), R.shape)
        st, nll, obj, _ = filtsmooth.linear_filtsmooth(setup.x0, dtm, (H, c, reg * eye / N))
        yield st, nll, obj, reg
        while True:
            nll_old, obj_old, st_old = nll, obj, st
            H, c, _ = linearize_at_previous_states(setup, st[0])
            st, nll, obj, _ = filtsmooth.linear_filtsmooth(setup.x0, dtm, (H, c, reg * eye / N))
            yield st, nll, obj, reg
            if crit(obj, obj_old, nll, nll_old, st[0], st_old[0], rtol=tau, atol=tau):
                reg *= reg_fact
                tau *= tau_fact
                if reg == 0:
                    break
                elif reg < reg_final:
                    reg = 0.0
                    tau = min(tau_final, 1e-5)
            if np.isnan(nll) or np.isnan(obj):
                break

    return gen(), setup


def linearize_regularized(setup, m, lam):
    """``observations.py:64-83`` at a batch of states: the EK1 rows
    (Jacobian H, offset = the residual itself, as the reference stacks
    ``res`` and not ``res - H m``) over the rows (I, -m) with noise chol
    blockdiag(0, I / sqrt(lam))."""
    d = setup.d
    D = m.shape[-1]
    y = filtsmooth.mv(setup.E0, m)
    H = setup.E1 - setup.ivp.jac(y) @ setup.E0
    res = filtsmooth.mv(setup.E1, m) - setup.ivp.f(None, y)
    lead = m.shape[:-1]
    full_H = np.concatenate([H, np.broadcast_to(np.eye(D), lead + (D, D))], axis=-2)
    full_b = np.concatenate([res, -m], axis=-1)
    R = np.zeros(lead + (d + D, d + D))
    R[..., d:, d:] = np.eye(D) / np.sqrt(lam)
    return full_H, full_b, R


def lm_ieks_iterator(setup, init_means, reg=1e0, nu=10.0):
    """``iterators.py:109-133``, Levenberg-Marquardt-regularized IEKS
    (arguments: the set-up's dtm, om and x0, and the trajectory to linearize
    at first, one state per step).  The reference's step-size adaptation
    (``nu``) is commented out, so reg stays fixed; the loop ends when nll and
    obj both stall (``jnp.isclose`` defaults rtol 1e-5, atol 1e-8) or on
    NaN.  Yields (states, nll, obj, reg)."""
    dtm = (setup.F, setup.QL)

    def gen():
        st, nll, obj, _ = filtsmooth.linear_filtsmooth(setup.x0, dtm, linearize_regularized(setup, init_means, reg))
        yield st, nll, obj, reg
        while True:
            nll_old, obj_old = nll, obj
            st, nll, obj, _ = filtsmooth.linear_filtsmooth(setup.x0, dtm,
                                                           linearize_regularized(setup, st[0][1:], reg))
            yield st, nll, obj, reg
            if (np.isclose(nll_old, nll) and np.isclose(obj_old, obj)) or np.isnan(nll) or np.isnan(obj):
                break

    return gen()
