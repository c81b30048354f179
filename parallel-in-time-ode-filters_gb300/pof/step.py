"""One IEKS iteration (pof/step.py)."""

import torch

from . import _lib
from .observations import AffineModel, linearize
from .parallel_filtsmooth import linear_filtsmooth as parallel_linear_filtsmooth
from .sequential_filtsmooth import linear_filtsmooth as sequential_linear_filtsmooth
from .utils import MVNSqrt


def _builtin_linearize(om, means):
    """EK1 of a built-in field at means[1:] in libpof."""
    setup = om.setup
    name, params = om.field
    n = means.shape[0] - 1
    D = means.shape[1]
    d = setup["iwp"].wiener_process_dimension
    dtype = means.dtype
    means = means.contiguous()
    H = torch.empty((n, d, D), dtype=dtype, device=means.device)
    c = torch.empty((n, d), dtype=dtype, device=means.device)
    p = torch.tensor(params if params else (0.0,), dtype=dtype, device=means.device)
    rc = _lib.lib().pof_linearize(_lib.dtype_code(dtype), n, D, d, _lib.FIELDS[name], _lib.ptr(p), float(setup["dt"]),
                                  _lib.ptr(means), _lib.ptr(H), _lib.ptr(c), _lib.stream_handle())
    _lib.check(rc, "pof_linearize")
    R = torch.zeros((n, d, d), dtype=dtype, device=means.device)
    return AffineModel(H, c, R)


def linearize_at_previous_states(om, prev_states):
    """EK1 of the residual model at states[1:] (pof/step.py:12-22)."""
    if getattr(om, "field", None) is not None and om.setup is not None:
        return _builtin_linearize(om, prev_states.mean)
    lin_traj = MVNSqrt(prev_states.mean[1:], prev_states.chol[1:])
    return linearize(om, lin_traj)


def inflate(state):
    """pof/step.py:25-30 (unused by the solver, kept for API parity)."""
    return MVNSqrt(state.mean, state.chol + torch.eye(state.chol.shape[-1], dtype=state.chol.dtype,
                                                      device=state.chol.device) * 1e-3)


def ieks_step(*, om, dtm, x0, states, calibrate=True, sequential=False):
    """Linearize at the previous states, filter + smooth, calibrate
    (pof/step.py:33-45).  Returns (states, nll, obj, ssq)."""
    dom = linearize_at_previous_states(om, states)
    if not sequential:
        states, nll, obj, ssq = parallel_linear_filtsmooth(x0, dtm, dom)
    else:
        states, nll, obj, ssq = sequential_linear_filtsmooth(x0, dtm, dom)
    if calibrate:
        states = MVNSqrt(states.mean, ssq**0.5 * states.chol)
    return states, nll, obj, ssq
