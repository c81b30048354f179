"""Primitives of the reference restated in NumPy float64 (test infrastructure).

All functions accept leading batch axes (``...``) where the reference uses
``jax.vmap``.
"""

import math

import numpy as np
import scipy.linalg as sla
import scipy.special


def T(a):
    """Swap the two trailing axes."""
    return np.swapaxes(a, -1, -2)


def tria(A):
    """Lower-triangular square root via QR: ``L L^T == A A^T``.

    Follows ``pof/utils.py:33-41``: ``qr(A.T, mode="r").T`` with LAPACK's
    Householder QR (``dgeqrf``; numpy's ``linalg.qr`` calls it).  The diagonal
    signs are LAPACK's: ``R_jj = -sign(alpha_j) * norm`` (``dlarfg``).
    """
    return T(np.linalg.qr(T(A), mode="r"))


def solve_tri(L, B, lower=True, trans=False):
    """``jax.scipy.linalg.solve_triangular`` restated (batched)."""
    return sla.solve_triangular(L, B, lower=lower, trans=1 if trans else 0)


def mvn_loglikelihood(x, chol_cov):
    """``pof/utils.py:22-30``: log N(x; 0, L L^T) with lower-triangular L."""
    dim = chol_cov.shape[-1]
    y = solve_tri(chol_cov, x[..., None], lower=True)[..., 0]
    diag = np.diagonal(chol_cov, axis1=-2, axis2=-1)
    normalizing_constant = np.sum(np.log(np.abs(diag)), -1) + dim * np.log(2 * np.pi) / 2.0
    norm_y = np.sum(y * y, -1)
    return -0.5 * norm_y - normalizing_constant


def whiten(m, cholP):
    """``pof/utils.py:110-112``: ``solve_triangular(cholP.T, m)`` with the
    default ``lower=False``, i.e. ``cholP^{-T} m`` (quirk: not ``cholP^{-1} m``)."""
    return solve_tri(T(cholP), m[..., None], lower=False)[..., 0]


def objective_function_value(mnext, m, F, QL):
    """``pof/utils.py:97-101``: ``|| QL^{-1} (mnext - F m) ||^2``."""
    r = mnext - (F @ m[..., None])[..., 0]
    r = solve_tri(QL, r[..., None], lower=True)[..., 0]
    return np.sum(r * r, -1)


def append_zeros_along_new_axis(z, N):
    """``pof/utils.py:93-94``."""
    return np.concatenate([z[None], np.zeros((N,) + z.shape)])


# --------------------------------------------------------------------------
# IWP prior, ``pof/transitions.py``
# --------------------------------------------------------------------------


def preconditioned_discretize_1d(q):
    """``pof/transitions.py:37-41``: A = flip(lower Pascal), L = chol(flip(Hilbert))."""
    A = np.flip(scipy.linalg.pascal(q + 1, kind="lower", exact=False))
    Q = np.flip(scipy.linalg.hilbert(q + 1))
    return np.ascontiguousarray(A), np.linalg.cholesky(np.ascontiguousarray(Q))


def preconditioned_discretize(d, q):
    """``pof/transitions.py:44-50``: I_d (x) A_1d and I_d (x) L_1d (independent of h)."""
    A1, L1 = preconditioned_discretize_1d(q)
    I = np.eye(d)
    return np.kron(I, A1), np.kron(I, L1)


def nordsieck_preconditioner_1d(q, dt):
    """``pof/transitions.py:53-61``: diag(|h|^(q-i+1/2) / (q-i)!) and its inverse."""
    powers = np.arange(q, -1, -1)
    scales = scipy.special.factorial(powers)
    powers = powers + 0.5
    s = (abs(dt) ** powers) / scales
    si = (abs(dt) ** (-powers)) * scales
    return np.diag(s), np.diag(si)


def nordsieck_preconditioner(d, q, dt):
    """``pof/transitions.py:64-68``."""
    P, PI = nordsieck_preconditioner_1d(q, dt)
    I = np.eye(d)
    return np.kron(I, P), np.kron(I, PI)


def non_preconditioned_discretize(d, q, dt):
    """``pof/transitions.py:71-77``: (P A PI, P L_Q)."""
    P, PI = nordsieck_preconditioner(d, q, dt)
    F, QL = preconditioned_discretize(d, q)
    return P @ F @ PI, P @ QL


def projection_matrix(d, q, k):
    """``pof/transitions.py:80-88``: I_d (x) e_k^T."""
    return np.kron(np.eye(d), np.eye(1, q + 1, k))


def discretize_transitions(d, q, steps):
    """``pof/transitions.py:96-100`` (``steps`` given explicitly)."""
    Fs, QLs = zip(*[non_preconditioned_discretize(d, q, float(h)) for h in steps])
    return np.stack(Fs), np.stack(QLs)


def factorial(n):
    return float(math.factorial(n))
