"""IWP prior in Nordsieck-preconditioned coordinates (pof/transitions.py).

Small (D x D) set-up matrices, built in float64 on the host and placed on
the requested device.
"""

import math
from typing import Any, NamedTuple

import numpy as np
import scipy.linalg
import torch

from .utils import default_device


class TransitionModel(NamedTuple):
    """x' | x ~ N(F x, QL QL^T) (pof/transitions.py:15-19)."""

    F: Any
    QL: Any


class IWP(NamedTuple):
    """pof/transitions.py:22-24."""

    wiener_process_dimension: int
    num_derivatives: int


def _t(a, device=None, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=device or default_device())


def hilbert(n):
    return scipy.linalg.hilbert(n)


def pascal(n):
    return scipy.linalg.pascal(n, kind="lower", exact=False)


def _preconditioned_1d_np(q):
    A = np.flip(pascal(q + 1))
    Q = np.flip(hilbert(q + 1))
    return np.ascontiguousarray(A), np.linalg.cholesky(np.ascontiguousarray(Q))


def preconditioned_discretize_1d(iwp: IWP, device=None):
    """A = flip(lower Pascal), L = chol(flip(Hilbert)) (pof/transitions.py:37-41)."""
    A, L = _preconditioned_1d_np(iwp.num_derivatives)
    return _t(A, device), _t(L, device)


def preconditioned_discretize(iwp: IWP, device=None):
    """I_d (x) A_1d, I_d (x) L_1d -- independent of the step (pof/transitions.py:44-50)."""
    A, L = _preconditioned_1d_np(iwp.num_derivatives)
    I = np.eye(iwp.wiener_process_dimension)
    return _t(np.kron(I, A), device), _t(np.kron(I, L), device)


def _nordsieck_1d_np(q, dt):
    powers = np.arange(q, -1, -1)
    scales = np.array([math.factorial(int(p)) for p in powers], dtype=np.float64)
    powers = powers + 0.5
    s = (abs(float(dt)) ** powers) / scales
    si = (abs(float(dt)) ** (-powers)) * scales
    return np.diag(s), np.diag(si)


def nordsieck_preconditioner_1d(iwp: IWP, dt, device=None):
    """diag(|h|^(q-i+1/2)/(q-i)!) and its inverse (pof/transitions.py:53-61)."""
    P, PI = _nordsieck_1d_np(iwp.num_derivatives, dt)
    return _t(P, device), _t(PI, device)


def nordsieck_preconditioner(iwp: IWP, dt, device=None):
    """pof/transitions.py:64-68."""
    P, PI = _nordsieck_1d_np(iwp.num_derivatives, dt)
    I = np.eye(iwp.wiener_process_dimension)
    return _t(np.kron(I, P), device), _t(np.kron(I, PI), device)


def non_preconditioned_discretize(iwp: IWP, dt, device=None):
    """(P A PI, P L_Q) (pof/transitions.py:71-77)."""
    P, PI = _nordsieck_1d_np(iwp.num_derivatives, dt)
    A, L = _preconditioned_1d_np(iwp.num_derivatives)
    I = np.eye(iwp.wiener_process_dimension)
    P, PI, A, L = (np.kron(I, x) for x in (P, PI, A, L))
    return _t(P @ A @ PI, device), _t(P @ L, device)


def projection_matrix_1d(iwp: IWP, derivative_to_project_onto, device=None):
    """pof/transitions.py:80-82."""
    return _t(np.eye(1, iwp.num_derivatives + 1, derivative_to_project_onto), device)


def projection_matrix(iwp: IWP, derivative_to_project_onto, device=None):
    """I_d (x) e_k^T (pof/transitions.py:85-88)."""
    e = np.eye(1, iwp.num_derivatives + 1, derivative_to_project_onto)
    return _t(np.kron(np.eye(iwp.wiener_process_dimension), e), device)


def get_transition_model(iwp: IWP, dt, device=None):
    """pof/transitions.py:91-93."""
    return TransitionModel(*non_preconditioned_discretize(iwp, dt, device))


def discretize_transitions(iwp: IWP, times=None, steps=None, device=None):
    """Per-step non-preconditioned transitions (pof/transitions.py:96-100)."""
    if steps is None:
        times = np.asarray(times.cpu() if isinstance(times, torch.Tensor) else times, dtype=np.float64)
        steps = times[1:] - times[:-1]
    steps = np.asarray(steps.cpu() if isinstance(steps, torch.Tensor) else steps, dtype=np.float64)
    Fs, QLs = zip(*[non_preconditioned_discretize(iwp, float(h), device=torch.device("cpu")) for h in steps])
    dev = device or default_device()
    return TransitionModel(torch.stack(Fs).to(dev), torch.stack(QLs).to(dev))
