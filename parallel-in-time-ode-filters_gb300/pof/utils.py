"""Small helpers of pof/utils.py, on torch tensors (any device).

These are set-up and convenience helpers; the filter/smoother hot path runs
in libpof (see ``pof.parallel_filtsmooth``).
"""

import math
from typing import Any, NamedTuple

import torch


class MVNSqrt(NamedTuple):
    """Gaussian in square-root form (pof/utils.py:9-11)."""

    mean: Any
    chol: Any


class AffineModel(NamedTuple):
    """x -> A x + b (pof/utils.py:14-19)."""

    A: Any
    b: Any

    def __call__(self, x):
        return self.A @ x + self.b


def default_device():
    if not torch.cuda.is_available():
        raise RuntimeError("pof needs a CUDA device (the solver runs in libpof on the GPU)")
    return torch.device("cuda", torch.cuda.current_device())


def as_tensor(x, dtype=torch.float64, device=None):
    device = device or default_device()
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype)
    return torch.as_tensor(x, dtype=dtype, device=device)


def tria(A):
    """Lower-triangular square root, qr(A^T, mode='r')^T (pof/utils.py:33-35)."""
    return qr(A.transpose(-1, -2)).transpose(-1, -2)


def qr(A):
    """R factor of A (pof/utils.py:38-41)."""
    return torch.linalg.qr(A, mode="r")[1]


def mvn_loglikelihood(x, chol_cov):
    """log N(x; 0, L L^T) (pof/utils.py:22-30)."""
    dim = chol_cov.shape[-1]
    y = torch.linalg.solve_triangular(chol_cov, x.unsqueeze(-1), upper=False).squeeze(-1)
    diag = torch.diagonal(chol_cov, dim1=-2, dim2=-1)
    normalizing_constant = torch.log(diag.abs()).sum(-1) + dim * math.log(2 * math.pi) / 2.0
    return -0.5 * (y * y).sum(-1) - normalizing_constant


def whiten(m, cholP):
    """solve_triangular(cholP^T, m) with upper=True, i.e. cholP^{-T} m (pof/utils.py:110-112)."""
    return torch.linalg.solve_triangular(cholP.transpose(-1, -2), m.unsqueeze(-1), upper=True).squeeze(-1)


def objective_function_value(mnext, m, transition_model):
    """|| QL^{-1} (mnext - F m) ||^2 (pof/utils.py:97-101)."""
    F, QL = transition_model
    r = mnext - (F @ m.unsqueeze(-1)).squeeze(-1)
    r = torch.linalg.solve_triangular(QL, r.unsqueeze(-1), upper=False).squeeze(-1)
    return (r * r).sum(-1)


def append_zeros_along_new_axis(z, N):
    """pof/utils.py:93-94."""
    return torch.cat([z[None], torch.zeros((N,) + tuple(z.shape), dtype=z.dtype, device=z.device)])


def _gmul(A, x: MVNSqrt):
    """A * x for a Gaussian (pof/utils.py:104-107)."""
    return MVNSqrt(A @ x.mean, A @ x.chol)


def gmul_stack(A, states: MVNSqrt):
    """vmap(_gmul, in_axes=[None, 0])(A, states)."""
    return MVNSqrt(states.mean @ A.transpose(-1, -2), A @ states.chol)
