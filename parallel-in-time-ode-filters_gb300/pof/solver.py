"""Drop-in solver API (pof/solver.py)."""

import torch

from . import _lib
from . import convergence_criteria
from .convenience import get_initial_trajectory, set_up_solver, set_up_solver_no_precond
from .sequential_filtsmooth import filtsmooth as seq_fs
from .parallel_filtsmooth import linear_filtsmooth as parallel_linear_filtsmooth
from .step import ieks_step
from .utils import MVNSqrt, gmul_stack


def _solve_builtin(setup, states, calibrate, maxiters, precision="float64", maxiters_f32=10_000, rtol_f32=1e-5,
                   settle_f32=float("inf"), sequential=False):
    """The whole IEKS loop in libpof (pof_ieks_solve): linearization, chunked
    filter/smoother, calibration and the convergence test all on the device.
    precision="mixed": float32 iterations first, float64 polish after
    (pof_ieks_solve_mixed).  sequential: the sequential filter/smoother in
    the loop (pof_ieks_solve_sequential)."""
    om = setup["om"]
    name, params = om.field
    x0 = setup["x0"]
    means = states.mean.to(torch.float64).contiguous().clone()
    N, D = means.shape
    n = N - 1
    d = setup["iwp"].wiener_process_dimension
    dev = means.device
    F = setup["dtm"].F[0].contiguous()
    QL = setup["dtm"].QL[0].contiguous()
    chols = torch.empty((N, D, D), dtype=torch.float64, device=dev)
    info = torch.zeros(_lib.I_COUNT, dtype=torch.float64, device=dev)
    p = torch.tensor(params if params else (0.0,), dtype=torch.float64, device=dev)
    lib = _lib.lib()
    m0 = x0.mean.contiguous()
    L0 = x0.chol.contiguous()
    if precision == "mixed":
        info = torch.zeros(_lib.I_COUNT + 2, dtype=torch.float64, device=dev)
        wsb = lib.pof_ieks_mixed_workspace_bytes(n, D, d)
        ws = _lib.workspace(wsb, dev)
        rc = lib.pof_ieks_solve_mixed(n, D, d, _lib.FIELDS[name], _lib.ptr(p), float(setup["dt"]), _lib.ptr(m0),
                                      _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL), _lib.ptr(means), _lib.ptr(chols),
                                      int(maxiters_f32), float(rtol_f32), float(settle_f32), int(maxiters),
                                      int(bool(calibrate)),
                                      _lib.ptr(info), _lib.ptr(ws), wsb, _lib.stream_handle())
        _lib.check(rc, "pof_ieks_solve_mixed")
    else:
        wsq = lib.pof_ieks_sequential_workspace_bytes if sequential else lib.pof_ieks_workspace_bytes
        entry = lib.pof_ieks_solve_sequential if sequential else lib.pof_ieks_solve
        wsb = wsq(_lib.POF_F64, n, D, d)
        ws = _lib.workspace(wsb, dev)
        rc = entry(_lib.POF_F64, n, D, d, _lib.FIELDS[name], _lib.ptr(p), float(setup["dt"]),
                   _lib.ptr(m0), _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL), _lib.ptr(means),
                   _lib.ptr(chols), int(maxiters), int(bool(calibrate)), _lib.ptr(info), _lib.ptr(ws),
                   wsb, _lib.stream_handle())
        _lib.check(rc, "pof_ieks_solve_sequential" if sequential else "pof_ieks_solve")
    info_dict = {
        "iterations": info[_lib.I_ITERATIONS].to(torch.int64),
        # the sequential twin reports +sum log-likelihood (quirk of
        # pof/sequential_filtsmooth/filter.py:23-30), the parallel filter -sum
        "nll": -info[_lib.I_NLL] if sequential else info[_lib.I_NLL],
        "obj": info[_lib.I_OBJ],
        "sigma_squared": info[_lib.I_SSQ],
        "status": info[_lib.I_STATUS].to(torch.int64),
        "calibrated": bool(calibrate),
    }
    if precision == "mixed":
        info_dict["iterations_float32"] = info[_lib.I_COUNT].to(torch.int64)
        info_dict["best_change_float32"] = info[_lib.I_COUNT + 1]
    return MVNSqrt(means, chols), info_dict


def solve(*, f, y0, ts, order, init="prior", calibrate=True, maxiters=10_000, sequential=False,
          precision="float64", maxiters_f32=10_000, rtol_f32=1e-5, settle_f32=float("inf"), rtol=1e-6, stop=None):
    """Parallel-in-time IEKS (pof/solver.py:11-73).

    Returns (MVNSqrt(means (N, d), chol_covs (N, d, D)), info) with
    info = {iterations, nll, obj, sigma_squared, status, calibrated}
    (status: why the loop stopped, 0 converged, 1 maxiters, 2 non-finite).
    Built-in fields (pof.ivp) run the whole loop on the device, with the
    parallel or (sequential=True) the sequential filter/smoother; other
    torch vector fields are linearized with torch.func on the device and
    filtered/smoothed by libpof, with the loop test read back each
    iteration.

    precision="mixed" (built-in fields, an addition to the reference's
    signature): float32 IEKS iterations until the objective's relative change
    is below rtol_f32, then float64 iterations to the reference's criterion;
    info["iterations"] counts the float64 ones, info["iterations_float32"]
    the others.

    rtol: the objective tolerance of crit (pof/convergence_criteria.py:4-13,
    the reference's 1e-6; the device loops take the reference's value).
    stop: a callable checked before every iteration of the host-driven loops
    (fields without a device loop at their shape); once it returns True the
    loop ends with the last iterate and info["status"] 3 (cancelled)."""
    setup = set_up_solver(f=f, y0=y0, ts=ts, order=order)
    om = setup["om"]
    x0 = setup["x0"]
    states = get_initial_trajectory(setup, method=init)

    builtin = (om.field is not None and om.field[0] not in _lib.DENSE_FIELDS
               and _lib.shape_supported(x0.mean.shape[0], setup["iwp"].wiener_process_dimension))
    if builtin and (not sequential or precision == "float64"):
        states, info_dict = _solve_builtin(setup, states, calibrate, maxiters, precision, maxiters_f32, rtol_f32,
                                           settle_f32, sequential=sequential)
        return gmul_stack(setup["E0"], states), info_dict
    if precision == "mixed" and om.field is not None and not sequential:
        # fields without a device loop at this shape (the dense path's):
        # the same float32 phase and float64 polish, driven from the host
        means, it32, best = _float32_phase(setup, states, maxiters_f32, rtol_f32, settle_f32, stop)
        out, info_dict = _solve_loop(setup, MVNSqrt(means, states.chol), calibrate, maxiters, sequential, rtol, stop)
        info_dict["iterations_float32"] = torch.tensor(it32)
        info_dict["best_change_float32"] = torch.tensor(best, dtype=torch.float64)
        return out, info_dict
    if precision != "float64":
        raise NotImplementedError("precision=%r needs a built-in field (pof.ivp)" % (precision,))
    return _solve_loop(setup, states, calibrate, maxiters, sequential, rtol, stop)


def _wait(dev):
    """Wait for this thread's current stream before a host read (the wait
    releases the GIL, so other host threads run meanwhile)."""
    if dev.type == "cuda":
        torch.cuda.current_stream(dev).synchronize()


def _float32_phase(setup, states, maxiters_f32, rtol_f32, settle_f32, stop=None):
    """The float32 iterations of pof_ieks_solve_mixed, driven from the host
    (for fields the device loops do not take, e.g. the dense path's): each
    linearizes in float64 at the current trajectory, scales every observation
    row to unit norm (the same constraint, a smaller range), filters and
    smooths in float32 and converts the means back; a non-finite iterate is
    dropped.  The phase ends when the largest change of y = E0 m falls below
    rtol_f32 relative to max |y|, after three changes that did not shrink
    once the smallest change is below settle_f32, or after maxiters_f32
    iterations; a phase whose smallest change never came within 100 rtol_f32
    is discarded.  Returns (float64 means, kept iterations, smallest change)."""
    from .step import linearize_at_previous_states

    dtm, om, x0 = setup["dtm"], setup["om"], setup["x0"]
    E0 = setup["E0"]
    F, QL = dtm.F, dtm.QL
    if F.dim() == 3 and F.stride(0) == 0 and QL.stride(0) == 0:
        F, QL = F[0], QL[0]  # one pair broadcast over the steps: convert it once
    dtm32 = (F.to(torch.float32), QL.to(torch.float32))
    x032 = MVNSqrt(x0.mean.to(torch.float32), x0.chol.to(torch.float32))
    means = states.mean.to(torch.float64)
    keep = means
    it32, prev, best, worse = 0, float("inf"), float("inf"), 0
    while it32 < maxiters_f32:
        if stop is not None and stop():
            break
        dom = linearize_at_previous_states(om, MVNSqrt(means, states.chol))
        inv = 1.0 / torch.linalg.vector_norm(dom.H, dim=-1)
        inv = torch.where(torch.isfinite(inv), inv, torch.ones_like(inv))
        H32 = (dom.H * inv[..., None]).to(torch.float32)
        c32 = (dom.b * inv).to(torch.float32)
        out, _, _, _ = parallel_linear_filtsmooth(x032, dtm32, (H32, c32, None))
        cand = out.mean.to(torch.float64)
        _wait(cand.device)
        if not bool(torch.isfinite(cand).all()):
            break
        y_new, y_old = cand @ E0.T, means @ E0.T
        dy = float((y_new - y_old).abs().max())
        ay = float(y_old.abs().max())
        it32 += 1
        means = cand
        rel = dy / ay if ay > 0 else dy
        best = min(best, rel)
        if rel < rtol_f32:
            break
        worse = worse + 1 if (rel >= prev and best < settle_f32) else (worse if rel >= prev else 0)
        if worse >= 3:
            break
        prev = rel
    if it32 > 0 and not best < 100.0 * rtol_f32:
        return keep, 0, best
    return means, it32, best


def _solve_loop(setup, states, calibrate, maxiters, sequential, rtol=1e-6, stop=None):
    """The IEKS loop of pof/solver.py:24-73 in Python: each iteration
    linearizes (libpof for built-in fields, torch.func otherwise) and runs
    libpof's filter/smoother; crit is read back each iteration."""
    dtm, om, x0 = setup["dtm"], setup["om"], setup["x0"]
    dev = x0.mean.device
    z = torch.zeros((), dtype=torch.float64, device=dev)
    nll = obj = ssq = z
    states_old, nll_old, obj_old = states, z, z
    k = 0
    conv = False
    cancelled = False
    while True:
        # cond (solver.py:36-45)
        if k >= 1:
            _wait(dev)
            conv = bool(convergence_criteria.crit(obj, obj_old, nll, nll_old, states, states_old, rtol=rtol))
        if not (k < 1 or (not conv and k <= maxiters)):
            break
        if stop is not None and stop():
            cancelled = True
            break
        # body (solver.py:47-55)
        states_old, nll_old, obj_old = states, nll, obj
        states, nll, obj, ssq = ieks_step(om=om, dtm=dtm, x0=x0, states=states_old, sequential=sequential)
        k += 1
    # the stopping reason (POF_SOLVE_*), as libpof's loop reports it
    finite = bool(torch.isfinite(torch.as_tensor(obj)).item() and torch.isfinite(torch.as_tensor(nll)).item())
    status = 3 if cancelled else (0 if (finite and conv) else (1 if finite else 2))
    info_dict = {"iterations": torch.tensor(k), "nll": nll, "obj": obj, "sigma_squared": ssq,
                 "status": torch.tensor(status), "calibrated": False}
    if calibrate:
        states = MVNSqrt(states.mean, ssq**0.5 * states.chol)
        info_dict["calibrated"] = True
    return gmul_stack(setup["E0"], states), info_dict


def solve_nonuniform(*, f, y0, ts, order, init="constant", calibrate=True, maxiters=10_000, sequential=False):
    """Parallel-in-time IEKS on a grid with its own step sizes (an addition
    to the reference, whose solve takes every step as ts[1] - ts[0],
    pof/convenience.py:14-16).  The set-up is the reference's
    set_up_solver_no_precond (pof/convenience.py:48-73): one
    non-preconditioned IWP transition per step, plain projections; the loop
    and the returned values are those of solve (pof/solver.py:24-73).  The
    per-step transitions go to libpof as (n, D, D) stacks."""
    setup = set_up_solver_no_precond(f=f, y0=y0, ts=ts, order=order)
    states = get_initial_trajectory(setup, method=init)
    return _solve_loop(setup, states, calibrate, maxiters, sequential)


def sequential_eks_solve(*, f, y0, ts, order, return_full_states=False, calibrate=True):
    """One extended Kalman smoother pass (pof/solver.py:76-96)."""
    setup = set_up_solver(f=f, y0=y0, ts=ts, order=order)
    states, nll, obj, ssq = seq_fs(setup["x0"], setup["dtm"], setup["om"])
    info_dict = {"nll": nll, "obj": obj, "sigma_squared": ssq, "calibrated": False}
    if calibrate:
        states = MVNSqrt(states.mean, ssq**0.5 * states.chol)
        info_dict["calibrated"] = True
    M = setup["P"] if return_full_states else setup["E0"]
    return gmul_stack(M, states), info_dict
