"""Sequential square-root filter (pof/sequential_filtsmooth/filter.py).

``extended_kalman_filter`` / ``linear_noiseless_filter`` run whole
trajectories in libpof on one GPU thread; ``_sqrt_predict`` and
``_sqrt_update`` are the one-step helpers, in torch, used by the
initialisation routines."""

import torch

from ..utils import MVNSqrt, mvn_loglikelihood, tria, whiten
from . import _call


def extended_kalman_filter(x0, discrete_transition_models, continuous_observation_model):
    """EKF linearizing at each predicted mean (filter.py:9-30): (filtered, ell, ssq)."""
    out, ell, _, ssq = _call.sequential(x0, discrete_transition_models, om=continuous_observation_model, smooth=False)
    return out, ell, ssq


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
