"""Small helpers of pof/utils.py, on torch tensors (any device).

These are set-up and convenience helpers; the filter/smoother hot path runs
in libpof (see ``pof.parallel_filtsmooth``).
"""

import math
import threading
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


def linearize(f, x):
    """First-order Taylor model of f at x: AffineModel(J, f(x) - J x), J by
    forward-mode differentiation (pof/utils.py:86-90)."""
    J = torch.func.jacfwd(f)(x)
    return AffineModel(J, f(x) - J @ x)


def _cholesky_update(chol, update_vector, multiplier=1.0):
    """Lower-triangular L' with L' L'^T = L L^T + multiplier v v^T, column by
    column (Krause and Igel, 2015, Algorithm 3.1, as pof/utils.py:123-172
    states it): omega starts at v and b at 1; for column j,
        L'_jj = sqrt(L_jj^2 + multiplier / b * omega_j^2),
        gamma = L_jj^2 b + multiplier omega_j^2,
        omega <- omega - (omega_j / L_jj) L[:, j],
        L'[:, j] = L'_jj (L[:, j] / L_jj + multiplier omega_j / gamma * omega),
        b <- b + multiplier (omega_j / L_jj)^2;
    then the strict upper triangle is zeroed and non-finite entries set to 0."""
    n = chol.shape[-1]
    omega = update_vector.clone()
    b = torch.ones((), dtype=chol.dtype, device=chol.device)
    cols, diag = [], []
    for j in range(n):
        ljj = chol[j, j]
        wj = omega[j]
        new_d = torch.sqrt(ljj * ljj + multiplier / b * wj * wj)
        gamma = ljj * ljj * b + multiplier * wj * wj
        col = chol[:, j]
        omega = omega - (wj / ljj) * col
        cols.append(new_d * (col / ljj + (multiplier * wj / gamma) * omega))
        diag.append(new_d)
        b = b + multiplier * (wj / ljj) ** 2
    out = torch.stack(cols, dim=1)
    out = torch.tril(out, -1) + torch.diag(torch.stack(diag))
    return torch.where(torch.isfinite(out), out, torch.zeros_like(out))


def cholesky_update_many(chol_init, update_vectors, multiplier):
    """Successive rank-one updates of a Cholesky factor by the rows of
    update_vectors (pof/utils.py:115-120)."""
    chol = chol_init
    for v in update_vectors:
        chol = _cholesky_update(chol, v, multiplier=multiplier)
    return chol


# torch.func.jvp enters forward-AD dual levels through a process-wide level
# counter, so two host threads in a jvp at once break each other's level
# ("no level exists").  The Taylor-mode initial values (the only forward AD
# the server's threads run) hold this lock.
FORWARD_AD_LOCK = threading.RLock()
