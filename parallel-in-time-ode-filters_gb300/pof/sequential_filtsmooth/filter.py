"""Sequential square-root filter (pof/sequential_filtsmooth/filter.py).

``extended_kalman_filter`` / ``linear_noiseless_filter`` run whole
trajectories in libpof on one GPU thread (built-in vector fields are
linearized inside the kernel); the EKF of any other torch vector field runs
step after step in torch (each step's linearization needs the previous
step's prediction).  ``_sqrt_predict`` and ``_sqrt_update`` are the one-step
helpers, in torch, also used by the initialisation routines."""

import torch

from ..observations import linearize
from ..utils import MVNSqrt, mvn_loglikelihood, tria, whiten
from . import _call


def extended_kalman_filter(x0, discrete_transition_models, continuous_observation_model):
    """EKF linearizing at each predicted mean (filter.py:9-30): (filtered, ell, ssq)."""
    if getattr(continuous_observation_model, "field", None) is None:
        return _ekf_steps(x0, discrete_transition_models, continuous_observation_model)
    out, ell, _, ssq = _call.sequential(x0, discrete_transition_models, om=continuous_observation_model, smooth=False)
    return out, ell, ssq


def _ekf_steps(x0, discrete_transition_models, om):
    """The EKF recursion of filter.py:9-30 in torch, one step after the
    other: predict, EK1 of `om` at the predicted state, update; ell summed,
    ssq averaged over the steps."""
    F, QL = discrete_transition_models
    n = F.shape[0]
    x = MVNSqrt(x0.mean, x0.chol)
    ms, Ls = [x.mean], [x.chol]
    ell = ssq = torch.zeros((), dtype=x.mean.dtype, device=x.mean.device)
    for k in range(n):
        x = _sqrt_predict(F[k], QL[k], x)
        H, b, R = linearize(om, x)
        x, ell_k, ssq_k = _sqrt_update(H, R, b, x)
        ell = ell + ell_k
        ssq = ssq + ssq_k
        ms.append(x.mean)
        Ls.append(x.chol)
    return MVNSqrt(torch.stack(ms), torch.stack(Ls)), ell, ssq / n


def linear_noiseless_filter(x0, discrete_transition_models, discrete_observation_models):
    """Linear sequential filter (filter.py:33-56): (filtered, ell, ssq)."""
    out, ell, _, ssq = _call.sequential(x0, discrete_transition_models, dom=discrete_observation_models, smooth=False)
    return out, ell, ssq


def _sqrt_predict(F, cholQ, x):
    """filter.py:59-66 (batched over leading axes)."""
    m, cholP = x
    m = (F @ m.unsqueeze(-1)).squeeze(-1)
    cholP = tria(torch.cat([F @ cholP, cholQ], dim=-1))
    return MVNSqrt(m, cholP)


def _sqrt_update(H, cholR, c, x):
    """filter.py:69-92."""
    m, cholP = x
    nx = m.shape[-1]
    ny = c.shape[-1]
    y_hat = H @ m + c
    y_diff = 0 - y_hat
    Z = torch.zeros((nx, ny), dtype=m.dtype, device=m.device)
    M = torch.cat([torch.cat([H @ cholP, cholR], 1), torch.cat([cholP, Z], 1)], 0)
    chol_S = tria(M)
    cholP = chol_S[ny:, ny:]
    G = chol_S[ny:, :ny]
    I = chol_S[:ny, :ny]
    wres = whiten(y_diff, I)
    ssq = (wres @ wres) / ny
    m = m + G @ torch.linalg.solve_triangular(I, y_diff.unsqueeze(-1), upper=False).squeeze(-1)
    ell = mvn_loglikelihood(y_diff, I)
    return MVNSqrt(m, cholP), ell, ssq
