"""Solver set-up (pof/convenience.py)."""

import torch

from . import initialization as init
from .observations import NonlinearModel, linearize
from .transitions import (
    IWP,
    TransitionModel,
    get_transition_model,
    nordsieck_preconditioner,
    preconditioned_discretize,
    projection_matrix,
)
from .utils import MVNSqrt, default_device, gmul_stack


def linearize_observation_model(observation_model, trajectory):
    """vmap(linearize) over a trajectory (pof/convenience.py:9-10)."""
    return linearize(observation_model, trajectory)


def _ts(ts):
    return torch.as_tensor(ts, dtype=torch.float64).to(default_device())


def set_up_solver(*, f, y0, ts, order):
    """pof/convenience.py:13-45: preconditioned IWP prior, Nordsieck P/PI,
    projections E0 P and E1 P, the residual model E1 x - f(E0 x) and the
    Taylor-mode x0 (times PI).  The N-1 identical transition models are
    exposed as a stride-0 expand of one (D, D) pair."""
    ts = _ts(ts)
    dts = ts[1:] - ts[:-1]
    dt = float(dts[0])  # uniform grid assumed, as in the reference (its check is commented out)
    y0 = torch.as_tensor(y0, dtype=torch.float64)
    d = y0.shape[0]
    n = ts.shape[0] - 1
    iwp = IWP(num_derivatives=order, wiener_process_dimension=d)
    A, QL = preconditioned_discretize(iwp)
    D = A.shape[0]
    dtm = TransitionModel(A.expand(n, D, D), QL.expand(n, D, D))
    P, PI = nordsieck_preconditioner(iwp, dt)
    E0, E1 = projection_matrix(iwp, 0), projection_matrix(iwp, 1)
    E0, E1 = E0 @ P, E1 @ P

    def om_fn(x, f=f, E0=E0, E1=E1):
        return E1 @ x - f(None, E0 @ x)

    setup = {
        "f": f,
        "y0": y0,
        "ts": ts,
        "dt": dt,
        "dtm": dtm,
        "E0": E0,
        "E1": E1,
        "P": P,
        "PI": PI,
        "order": order,
        "iwp": iwp,
    }
    om = NonlinearModel(om_fn, field=getattr(f, "pof_field", None), setup=setup)
    x0 = init.taylor_mode_init(f, y0, order)
    x0 = MVNSqrt(PI @ x0.mean, PI @ x0.chol)
    setup["om"] = om
    setup["x0"] = x0
    return setup


def set_up_solver_no_precond(*, f, y0, ts, order):
    """pof/convenience.py:48-73: per-step non-preconditioned transitions."""
    ts = _ts(ts)
    y0 = torch.as_tensor(y0, dtype=torch.float64)
    d = y0.shape[0]
    iwp = IWP(num_derivatives=order, wiener_process_dimension=d)
    steps = (ts[1:] - ts[:-1]).cpu()
    Fs, QLs = zip(*[get_transition_model(iwp, float(h)) for h in steps])
    dtm = TransitionModel(torch.stack(Fs), torch.stack(QLs))
    E0, E1 = projection_matrix(iwp, 0), projection_matrix(iwp, 1)

    def om_fn(x):
        return E1 @ x - f(None, E0 @ x)

    x0 = init.taylor_mode_init(f, y0, order)
    D = x0.mean.shape[0]
    I = torch.eye(D, dtype=torch.float64, device=x0.mean.device)
    return {"ts": ts, "dtm": dtm, "om": NonlinearModel(om_fn), "x0": x0, "E0": E0, "P": I, "PI": I,
            "order": order, "iwp": iwp, "f": f, "y0": y0}


def get_initial_trajectory(setup, method="prior"):
    """pof/convenience.py:76-92 ("prior" keeps the reference's behaviour: no PI)."""
    f, y0, order = setup["f"], setup["y0"], setup["order"]
    ts = setup["ts"]
    PI = setup["PI"]
    if method == "coarse":
        states = init.coarse_ekf_init(y0=y0, order=order, ts=ts, f=f, N=100)
        return gmul_stack(PI, states)
    elif method == "constant":
        states = init.constant_init(y0=y0, order=order, ts=ts, f=f)
        return gmul_stack(PI, states)
    elif method == "prior":
        return init.prior_init(f=f, y0=y0, order=order, ts=ts)
    else:
        raise Exception(f"method={method} not found")
