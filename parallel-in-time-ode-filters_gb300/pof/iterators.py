"""Host-side IEKS iterators (pof/iterators.py)."""

import torch

from . import convergence_criteria
from . import initialization as init
from .convenience import get_initial_trajectory, set_up_solver
from .observations import AffineModel, linearize, linearize_regularized
from .parallel_filtsmooth import linear_filtsmooth
from .step import ieks_step, linearize_at_previous_states
from .utils import MVNSqrt

fs = linear_filtsmooth


def lom(om, traj):
    """EK1 of the observation model at every state of a trajectory
    (pof/iterators.py:14: jit(vmap(linearize)))."""
    return linearize(om, traj)


def lom_reg(om, traj, reg):
    """Levenberg-Marquardt-regularized linearization at every state of a
    trajectory (pof/iterators.py:15-17: jit(vmap(linearize_regularized)))."""
    outs = [linearize_regularized(om, MVNSqrt(traj.mean[k], traj.chol[k]), reg) for k in range(traj.mean.shape[0])]
    return AffineModel(*(torch.stack(z) for z in zip(*outs)))


def ieks_iterator(*, f, y0, ts, order, init="prior"):
    """Generator of IEKS iterations until ``crit`` (pof/iterators.py:20-24)."""
    setup = set_up_solver(f=f, y0=y0, ts=ts, order=order)
    states = get_initial_trajectory(setup, method=init)
    return _ieks_iterator(setup["dtm"], setup["om"], setup["x0"], states), setup


def _ieks_iterator(dtm, om, x0, init_traj):
    """pof/iterators.py:27-41."""
    states, nll, obj, ssq = ieks_step(om=om, dtm=dtm, x0=x0, states=init_traj)
    yield states, nll, obj, ssq
    while True:
        nll_old, obj_old, states_old = nll, obj, states
        states, nll, obj, ssq = ieks_step(om=om, dtm=dtm, x0=x0, states=states_old)
        yield states, nll, obj, ssq
        if bool(convergence_criteria.crit(obj, obj_old, nll, nll_old, states, states_old)):
            break


def _with_R(dom, cholR):
    return AffineModel(dom.H, dom.b, cholR)


def qpm_ieks_iterator(*, f, y0, ts, order, init="prior", **kwargs):
    """Quadratic-penalty IEKS (pof/iterators.py:44-50)."""
    setup = set_up_solver(f=f, y0=y0, ts=ts, order=order)
    states = get_initial_trajectory(setup, method=init)
    return _qpm_ieks_iterator(setup["dtm"], setup["om"], setup["x0"], states, **kwargs), setup


def _qpm_ieks_iterator(dtm, om, x0, init_traj, reg_start=1e20, reg_final=1e-20, steps=40, tau_start=None,
                       tau_final=None):
    """pof/iterators.py:53-106: cholR = reg * I / N, reg and tau shrink geometrically."""
    N = dtm.F.shape[0]
    dom = linearize_at_previous_states(om, init_traj)
    reg_fact = (reg_final / reg_start) ** (1 / steps)
    if tau_start is None:
        tau_start, tau_final = 1e5, 1e-5
    tau_fact = (tau_final / tau_start) ** (1 / steps)
    reg, tau = reg_start, tau_start
    eye = torch.eye(dom.cholR.shape[-1], dtype=dom.cholR.dtype, device=dom.cholR.device).expand_as(dom.cholR)
    states, nll, obj, ssq = fs(x0, dtm, _with_R(dom, reg * eye / N))
    yield states, nll, obj, reg
    while True:
        nll_old, obj_old, states_old = nll, obj, states
        dom = linearize_at_previous_states(om, states)
        states, nll, obj, ssq = fs(x0, dtm, _with_R(dom, reg * eye / N))
        yield states, nll, obj, reg
        if bool(convergence_criteria.crit(obj, obj_old, nll, nll_old, states, states_old, rtol=tau, atol=tau)):
            reg *= reg_fact
            tau *= tau_fact
            if reg == 0:
                break
            elif reg < reg_final:
                reg = 0.0
                tau = min(tau_final, 1e-5)
        if bool(torch.isnan(nll)) or bool(torch.isnan(obj)):
            break


def lm_ieks_iterator(dtm, om, x0, init_traj, reg=1e0, nu=10.0):
    """Levenberg-Marquardt-regularized IEKS (pof/iterators.py:109-133)."""
    dom = lom_reg(om, init_traj, reg)
    out, nll, obj, ssq = fs(x0, dtm, dom)
    yield out, nll, obj, reg
    while True:
        nll_old, obj_old = nll, obj
        dom = lom_reg(om, MVNSqrt(out.mean[1:], out.chol[1:]), reg)
        out, nll, obj, ssq = fs(x0, dtm, dom)
        yield out, nll, obj, reg
        if (bool(torch.isclose(nll_old, nll)) and bool(torch.isclose(obj_old, obj))) or bool(torch.isnan(nll)) \
                or bool(torch.isnan(obj)):
            break
