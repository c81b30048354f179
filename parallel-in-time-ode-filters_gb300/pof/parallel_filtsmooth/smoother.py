"""Parallel square-root smoother (pof/parallel_filtsmooth/smoother.py).

``smoothing`` runs in libpof.  ``get_elements`` and
``sqrt_smoothing_operator`` are the reference's element construction and
associative operator, in torch on whatever device their inputs live, for
callers that build their own scans; libpof's kernels fuse both into the
chunked reverse scan."""

import torch

from ..utils import MVNSqrt, tria
from . import _call


def _sqrt_associative_params(transition_model, m, chol_P):
    """Smoother element (g, E, D) of one step, stacked over leading axes
    (pof/parallel_filtsmooth/smoother.py:37-50): Phi = tria([[F L, Q_L],
    [L, 0]]), E = (Phi11^-T Phi21^T)^T by a general (LU) solve as the
    reference's jnp.linalg.solve, g = m - E F m."""
    F, cholQ = transition_model
    nx = cholQ.shape[-1]
    Phi = torch.cat([torch.cat([F @ chol_P, cholQ], -1), torch.cat([chol_P, torch.zeros_like(cholQ)], -1)], -2)
    tp = tria(Phi)
    Phi11 = tp[..., :nx, :nx]
    Phi21 = tp[..., nx:, :nx]
    D = tp[..., nx:, nx:]
    E = torch.linalg.solve(Phi11.transpose(-1, -2), Phi21.transpose(-1, -2)).transpose(-1, -2)
    g = m - (E @ (F @ m.unsqueeze(-1))).squeeze(-1)
    return g, E, D


def get_elements(transition_models, filtering_trajectory):
    """The N - 1 smoother elements of a filtered trajectory and the terminal
    element (m_T, 0, L_T) (pof/parallel_filtsmooth/smoother.py:25-34)."""
    F, QL = transition_models
    ms, Ps = filtering_trajectory
    g, E, L = _sqrt_associative_params((F, QL), ms[:-1], Ps[:-1])
    g = torch.cat([g, ms[-1:]])
    E = torch.cat([E, torch.zeros_like(Ps[-1:])])
    L = torch.cat([L, Ps[-1:]])
    return g, E, L


def sqrt_smoothing_operator(elem1, elem2):
    """Combine smoother elements (g, E, D), elem1 later in time, stacked over
    leading axes (pof/parallel_filtsmooth/smoother.py:53-63):
    g = E2 g1 + g2, E = E2 E1, D = tria([E2 D1, D2])."""
    g1, E1, D1 = elem1
    g2, E2, D2 = elem2
    g = (E2 @ g1.unsqueeze(-1)).squeeze(-1) + g2
    E = E2 @ E1
    D = tria(torch.cat([E2 @ D1, D2], -1))
    return g, E, D


def smoothing(transition_models, filter_trajectory: MVNSqrt):
    """Smoothed states from filtered ones (pof/parallel_filtsmooth/smoother.py:8-22).
    Returns (MVNSqrt, obj)."""
    assert isinstance(filter_trajectory, MVNSqrt) or len(filter_trajectory) == 2
    return _call.smoothing(transition_models, MVNSqrt(*filter_trajectory))
