"""Parallel square-root filter (pof/parallel_filtsmooth/filter.py).

``linear_noiseless_filtering`` runs in libpof.  ``sqrt_filtering_operator``
is the reference's associative operator on filter elements, in torch on
whatever device its inputs live, for callers that build their own scans;
libpof's kernels fuse the same operator into the chunked scan."""

import torch

from ..utils import tria
from . import _call


def _mT(a):
    return a.transpose(-1, -2)


def _solve_lower(L, B, trans=False):
    """L^-1 B, or L^-T B with trans (jax.scipy.linalg.solve_triangular(L, B,
    lower=True, trans=trans))."""
    if trans:
        return torch.linalg.solve_triangular(_mT(L), B, upper=True)
    return torch.linalg.solve_triangular(L, B, upper=False)


def _mv(A, x):
    return (A @ x.unsqueeze(-1)).squeeze(-1)


def sqrt_filtering_operator(elem1, elem2):
    """Combine filter elements (A, b, U, eta, Z), elem1 earlier in time,
    stacked over leading axes (pof/parallel_filtsmooth/filter.py:117-142,
    vmapped there): Xi = tria([[U1^T Z2, I], [Z2, 0]]) and the products of
    the reference, in the same order."""
    A1, b1, U1, eta1, Z1 = elem1
    A2, b2, U2, eta2, Z2 = elem2
    nx = Z2.shape[-1]
    I = torch.eye(nx, dtype=Z2.dtype, device=Z2.device).expand(Z2.shape[:-2] + (nx, nx))
    Xi = torch.cat([torch.cat([_mT(U1) @ Z2, I], -1), torch.cat([Z2, torch.zeros_like(A1)], -1)], -2)
    tx = tria(Xi)
    Xi11 = tx[..., :nx, :nx]
    Xi21 = tx[..., nx:2 * nx, :nx]
    Xi22 = tx[..., nx:2 * nx, nx:]
    M = _solve_lower(Xi11, _mT(U1) @ _mT(A2))
    A = A2 @ A1 - _mT(M) @ _mT(Xi21) @ A1
    m = _solve_lower(Xi11, _mT(U1))
    b = _mv(A2 @ (I - _mT(m) @ _mT(Xi21)), b1 + _mv(U1 @ _mT(U1), eta2)) + b2
    U = tria(torch.cat([_mT(M), U2], -1))
    e = _solve_lower(Xi11, _mT(Xi21), trans=True)
    eta = _mv(_mT(A1) @ (I - _mT(e) @ _mT(U1)), eta2 - _mv(Z2 @ _mT(Z2), b1)) + eta1
    Z = tria(torch.cat([_mT(A1) @ Xi22, Z1], -1))
    return A, b, U, eta, Z


def linear_noiseless_filtering(x0, transition_models, observation_models):
    """Filtered states of a linear model with exact observations
    (pof/parallel_filtsmooth/filter.py:18-47), computed in libpof with the
    chunked associative scan.  Returns (MVNSqrt, nll, obj, ssq)."""
    out, nll, obj, ssq, _ = _call.filtsmooth("filter", x0, transition_models, observation_models)
    return out, nll, obj, ssq
