"""Sequential square-root RTS smoother (pof/sequential_filtsmooth/smoother.py)."""

import torch

from ..utils import MVNSqrt, objective_function_value, tria


def _sqrt_smooth(F, cholQ, xf, xs):
    """One RTS step (smoother.py:31-48), torch."""
    mf, cholPf = xf
    ms, cholPs = xs
    nx = F.shape[0]
    Phi = torch.cat([torch.cat([F @ cholPf, cholQ], 1), torch.cat([cholPf, torch.zeros_like(F)], 1)], 0)
    tria_Phi = tria(Phi)
    Phi11 = tria_Phi[:nx, :nx]
    Phi21 = tria_Phi[nx:, :nx]
    Phi22 = tria_Phi[nx:, nx:]
    gain = torch.linalg.solve_triangular(Phi11.T, Phi21.T, upper=True).T
    mean = mf + gain @ (ms - F @ mf)
    chol = tria(torch.cat([Phi22, gain @ cholPs], 1))
    return MVNSqrt(mean, chol)


def smoothing(discrete_transition_models, filter_trajectory):
    """Backward RTS pass over a filtered trajectory (smoother.py:8-28).

    Runs in libpof through the parallel smoother entry point (the smoothed
    marginals of a linear-Gaussian model do not depend on the bracketing)."""
    from ..parallel_filtsmooth import smoothing as psmooth

    return psmooth(discrete_transition_models, filter_trajectory)
