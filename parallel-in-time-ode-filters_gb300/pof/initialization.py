"""Initial state x0 and initial linearization trajectories
(pof/initialization.py).

Taylor-mode initialisation: the reference calls tornadox's TaylorMode
(``jax.experimental.jet``); here the derivatives come from nested
``torch.func.jvp``: with y_k(t) = sum_{j<k} y^(j) t^j / j!, the k-th
derivative of the solution at t0 is the (k-1)-th time derivative of
f(y_k(t)) at t0, which only involves y^(0..k-1).
"""

import math

import torch

from .sequential_filtsmooth.filter import _sqrt_predict
from .transitions import IWP, discretize_transitions
from .utils import FORWARD_AD_LOCK, MVNSqrt, default_device


def _nth_time_derivative(g, n):
    if n == 0:
        return g
    h = _nth_time_derivative(g, n - 1)

    def dh(t):
        return torch.func.jvp(h, (t,), (torch.ones_like(t),))[1]

    return dh


def taylor_derivatives(f, y0, num_derivatives):
    """(q+1, d) array of y^(k)(t0), k = 0..q, for y' = f(t, y) (time-independent f)."""
    y0 = torch.as_tensor(y0, dtype=torch.float64).detach().cpu()
    derivs = [y0]
    for k in range(1, num_derivatives + 1):
        coeffs = [dj / math.factorial(j) for j, dj in enumerate(derivs)]

        def g(t, coeffs=coeffs):
            y = coeffs[0] + 0 * t
            for j in range(1, len(coeffs)):
                y = y + coeffs[j] * t**j
            return f(None, y)

        derivs.append(_nth_time_derivative(g, k - 1)(torch.zeros((), dtype=torch.float64)).detach())
    return torch.stack(derivs)


def taylor_mode_init(f, y0, num_derivatives, device=None):
    """x0 = (y0, y0', ..., y0^(q)) per dimension, chol = 0 (pof/initialization.py:15-22)."""
    d = torch.as_tensor(y0).shape[0]
    with FORWARD_AD_LOCK:
        derivs = taylor_derivatives(f, y0, num_derivatives)  # (q+1, d)
    m0 = derivs.T.reshape(-1)
    D = d * (num_derivatives + 1)
    dev = device or default_device()
    return MVNSqrt(m0.to(dev), torch.zeros((D, D), dtype=torch.float64, device=dev))


def uncertain_init(f, y0, num_derivatives, var=1.0, device=None):
    """pof/initialization.py:25-39."""
    y0 = torch.as_tensor(y0, dtype=torch.float64)
    d = y0.shape[0]
    q = num_derivatives
    dy0 = f(None, y0).reshape(-1, 1)
    m0 = torch.cat([y0.reshape(-1, 1), dy0, torch.zeros((d, q - 1), dtype=torch.float64)], 1).reshape(-1)
    P0 = torch.eye(d * (q + 1), dtype=torch.float64) * var
    for j in range(d):
        P0[(q + 1) * j, (q + 1) * j] = 0
        P0[(q + 1) * j + 1, (q + 1) * j + 1] = 0
    dev = device or default_device()
    return MVNSqrt(m0.to(dev), torch.sqrt(P0).to(dev))


def constant_init(*, y0, order, ts, f=True, device=None):
    """[y0, f(y0), 0, ...] repeated, chol 0 (pof/initialization.py:42-56)."""
    y0 = torch.as_tensor(y0, dtype=torch.float64).cpu()
    d = y0.shape[-1]
    N = len(ts)
    dy0 = f(None, y0) if f is not None else torch.zeros_like(y0)
    x0 = torch.cat([y0[:, None], dy0[:, None], torch.zeros((d, order - 1), dtype=torch.float64)], dim=1)
    x0 = x0.reshape(1, -1)
    dev = device or default_device()
    traj = x0.to(dev).repeat(N, 1)
    D = traj.shape[1]
    return MVNSqrt(traj, torch.zeros((N, D, D), dtype=torch.float64, device=dev))


def classic_to_init(*, ys, order, f=None):
    """pof/initialization.py:59-72."""
    N, d = ys.shape
    if f is not None:
        dys = torch.func.vmap(lambda y: f(None, y))(ys)
    else:
        dys = torch.zeros_like(ys)
    traj = torch.cat([ys[:, :, None], dys[:, :, None], torch.zeros((N, d, order - 1), dtype=ys.dtype, device=ys.device)], 2)
    traj = traj.reshape(N, -1)
    D = traj.shape[1]
    return MVNSqrt(traj, torch.zeros((N, D, D), dtype=ys.dtype, device=ys.device))


def _prior_init(*, x0, dtm):
    """One-step predictions from x0 with every transition (pof/initialization.py:75-80)."""
    F, QL = dtm
    n = F.shape[0]
    m = x0.mean.expand(n, -1)
    L = x0.chol.expand(n, -1, -1)
    pm, pL = _sqrt_predict(F, QL, MVNSqrt(m, L))
    return MVNSqrt(torch.cat([x0.mean[None], pm]), torch.cat([x0.chol[None], pL]))


def prior_init(*, f, y0, order, ts, device=None):
    """pof/initialization.py:83-89: transitions at step sizes ts[1:] (absolute
    times, as in the reference), not preconditioned, result not scaled by PI.
    ``device``: where the trajectory is built (default: the current CUDA
    device)."""
    x0 = taylor_mode_init(f, y0, order, device=device)
    d = torch.as_tensor(y0).shape[0]
    iwp = IWP(num_derivatives=order, wiener_process_dimension=d)
    ts = torch.as_tensor(ts, dtype=torch.float64)
    dtm = discretize_transitions(iwp, steps=ts[1:], device=device)
    return _prior_init(x0=x0, dtm=dtm)


def updated_prior_init(*, x0, dtm, om):
    """pof/initialization.py:92-100."""
    from .observations import linearize
    from .sequential_filtsmooth.filter import _sqrt_update

    states = _prior_init(x0=x0, dtm=dtm)
    out_m, out_L = [], []
    for k in range(states.mean.shape[0]):
        x = MVNSqrt(states.mean[k], states.chol[k])
        H, b, cholR = linearize(om, x)
        (m, L), _, _ = _sqrt_update(H, cholR, b, x)
        out_m.append(m)
        out_L.append(L)
    return MVNSqrt(torch.stack(out_m), torch.stack(out_L))


def _get_coarse_dt(fine_ts):
    """pof/initialization.py:103-109."""
    T = float(fine_ts[-1] - fine_ts[0])
    N = len(fine_ts)
    return T / math.ceil(math.log2(N))


def coarse_ekf_init(*, f, y0, order, ts, N=10):
    """A sequential EKS on a coarse grid, sampled at floor(t / dt_coarse)
    (pof/initialization.py:112-129)."""
    from .solver import sequential_eks_solve

    ts = torch.as_tensor(ts, dtype=torch.float64)
    coarse_ts = torch.linspace(float(ts[0]), float(ts[-1]), N, dtype=torch.float64)
    coarse_dt = float(coarse_ts[1] - coarse_ts[0])
    out, _ = sequential_eks_solve(f=f, y0=y0, ts=coarse_ts, order=order, return_full_states=True)
    idxs = torch.floor(ts / coarse_dt).to(torch.long).to(out.mean.device)
    return MVNSqrt(out.mean[idxs], out.chol[idxs])
