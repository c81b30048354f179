"""Observation models and EK1 linearization (pof/observations.py).

``linearize`` of a user vector field uses ``torch.func.jacfwd`` (the
reference uses ``jax.jacfwd``), vectorized over time steps with
``torch.func.vmap`` on the device holding the states.  Built-in fields are
linearized inside libpof (``pof.step.linearize_at_previous_states``).
"""

from typing import Any, Callable, NamedTuple, Optional

import torch

from .transitions import IWP, projection_matrix
from .utils import MVNSqrt, tria


class NonlinearModel(NamedTuple):
    """y = f(x), noiseless (pof/observations.py:14-20).

    ``field`` optionally names a built-in vector field and ``setup`` holds the
    projections, so libpof can linearize on the device."""

    f: Callable
    field: Optional[tuple] = None
    setup: Any = None

    def __call__(self, x):
        return self.f(x)


class AffineModel(NamedTuple):
    """y = H x + b with noise chol cholR (pof/observations.py:23-32)."""

    H: Any
    b: Any
    cholR: Any


def _jac_and_value(f, m):
    def fx(x):
        v = f(x)
        return v, v

    J, v = torch.func.jacfwd(fx, has_aux=True)(m)
    return J, v


def linearize(f, x: MVNSqrt):
    """EK1 at the mean: H = df/dx, b = f(m) - H m, cholR = 0 (pof/observations.py:35-40).

    ``x.mean`` may carry leading batch axes; they are vectorized."""
    m = x.mean
    if m.dim() == 1:
        F_x, res = _jac_and_value(f, m)
    else:
        F_x, res = torch.func.vmap(lambda mm: _jac_and_value(f, mm))(m.reshape(-1, m.shape[-1]))
        F_x = F_x.reshape(m.shape[:-1] + F_x.shape[-2:])
        res = res.reshape(m.shape[:-1] + res.shape[-1:])
    d = res.shape[-1]
    cholR = torch.zeros(res.shape[:-1] + (d, d), dtype=m.dtype, device=m.device)
    b = res - (F_x @ m.unsqueeze(-1)).squeeze(-1)
    return AffineModel(F_x, b, cholR)


def uncertain_linearize(f, x: MVNSqrt):
    """WIP uncertainty-aware linearization (pof/observations.py:43-49)."""
    m, CL = x
    F_m, res = _jac_and_value(f, m)
    cholR = tria(F_m @ CL)
    return AffineModel(F_m, res - F_m @ m, cholR)


def linearize_ek0(f, x: MVNSqrt):
    """EK0: H = E1 (pof/observations.py:52-61)."""
    m = x.mean
    res = f(m)
    d = res.shape[0]
    q = (m.shape[0] // d) - 1
    E1 = projection_matrix(IWP(wiener_process_dimension=d, num_derivatives=q), 1, device=m.device).to(m.dtype)
    cholR = torch.zeros((d, d), dtype=m.dtype, device=m.device)
    return AffineModel(E1, res - E1 @ m, cholR)


def linearize_regularized(f, x: MVNSqrt, l):
    """EK1 stacked with a Tikhonov term (pof/observations.py:64-83)."""
    m = x.mean
    F_x, res = _jac_and_value(f, m)
    d, D = res.shape[0], m.shape[0]
    z = lambda *s: torch.zeros(s, dtype=m.dtype, device=m.device)  # noqa: E731
    reg_H = torch.eye(D, dtype=m.dtype, device=m.device)
    reg_b = -m
    reg_cholS = torch.eye(D, dtype=m.dtype, device=m.device) / (l**0.5)
    full_b = torch.cat([res, reg_b])
    full_H = torch.cat([F_x, reg_H], dim=0)
    full_cholR = torch.cat([torch.cat([z(d, d), z(d, D)], 1), torch.cat([z(D, d), reg_cholS], 1)], 0)
    return AffineModel(full_H, full_b, full_cholR)
