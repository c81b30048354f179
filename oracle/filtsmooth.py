"""Square-root Kalman filter/smoother, parallel and sequential (NumPy float64).

Test infrastructure.  Restates
``pof/parallel_filtsmooth/{__init__,filter,smoother}.py`` and
``pof/sequential_filtsmooth/{__init__,filter,smoother}.py``.

Array conventions (as in the reference): ``dtm = (F, QL)`` stacked over the
N-1 steps, ``dom = (H, c, cholR)`` stacked over the N-1 steps, ``x0 = (m0,
L0)``; states are ``(means (N,D), chols (N,D,D))``.
"""

import numpy as np

from .core import T, mvn_loglikelihood, objective_function_value, solve_tri, tria, whiten
from .scan import associative_scan, sequential_scan


def mv(A, x):
    return (A @ x[..., None])[..., 0]


# --------------------------------------------------------------------------
# parallel filter, pof/parallel_filtsmooth/filter.py
# --------------------------------------------------------------------------


def get_element(F, cholQ, H, c, cholR, ms, Ls):
    """``filter.py:50-81``: filter element (A, b, U, eta, Z) of one step."""
    nx = F.shape[-1]
    ny = c.shape[-1]
    batch = F.shape[:-2]
    m1 = mv(F, ms)
    N1_ = tria(np.concatenate((F @ Ls, cholQ), axis=-1))
    top = np.concatenate((H @ N1_, cholR), axis=-1)
    bot = np.concatenate((N1_, np.zeros(batch + (nx, ny))), axis=-1)
    TP = tria(np.concatenate((top, bot), axis=-2))
    Psi11 = TP[..., :ny, :ny]
    Psi21 = TP[..., ny:, :ny]
    U = TP[..., ny:, ny:]
    K = T(solve_tri(Psi11, T(Psi21), lower=True, trans=True))
    A = F - K @ H @ F
    b = m1 + mv(K, -mv(H, m1) - c)
    Z = T(solve_tri(Psi11, H @ F, lower=True))
    eta = mv(T(solve_tri(Psi11, T(Z), lower=True, trans=True)), -c)
    if nx > ny:
        Z = np.concatenate([Z, np.zeros(batch + (nx, nx - ny))], axis=-1)
    else:
        Z = tria(Z)
    return A, b, U, eta, Z


def sqrt_filtering_operator(elem1, elem2):
    """``filter.py:117-142``: combine (elem1 earlier, elem2 later)."""
    A1, b1, U1, eta1, Z1 = elem1
    A2, b2, U2, eta2, Z2 = elem2
    nx = Z2.shape[-1]
    batch = Z2.shape[:-2]
    I = np.broadcast_to(np.eye(nx), batch + (nx, nx))
    Xi = np.concatenate(
        (
            np.concatenate((T(U1) @ Z2, I), axis=-1),
            np.concatenate((Z2, np.zeros_like(A1)), axis=-1),
        ),
        axis=-2,
    )
    tx = tria(Xi)
    Xi11 = tx[..., :nx, :nx]
    Xi21 = tx[..., nx : nx + nx, :nx]
    Xi22 = tx[..., nx : nx + nx, nx:]
    M = solve_tri(Xi11, T(U1) @ T(A2), lower=True)
    A = A2 @ A1 - T(M) @ T(Xi21) @ A1
    m = solve_tri(Xi11, T(U1), lower=True)
    b = mv(A2 @ (I - T(m) @ T(Xi21)), b1 + mv(U1 @ T(U1), eta2)) + b2
    _U = T(solve_tri(Xi11, T(U1) @ T(A2), lower=True))
    U = tria(np.concatenate([_U, U2], axis=-1))
    _e = solve_tri(Xi11, T(Xi21), lower=True, trans=True)
    eta = mv(T(A1) @ (I - T(_e) @ T(U1)), eta2 - mv(Z2 @ T(Z2), b1)) + eta1
    Z = tria(np.concatenate([T(A1) @ Xi22, Z1], axis=-1))
    return A, b, U, eta, Z


def get_obs(F, cholQ, H, c, cholR, m, cholP):
    """``filter.py:84-93``: predicted observation mean and chol."""
    pm = mv(F, m)
    pc = tria(np.concatenate([F @ cholP, cholQ], axis=-1))
    obs_mean = mv(H, pm) + c
    obs_chol = tria(np.concatenate([H @ pc, cholR], axis=-1))
    return obs_mean, obs_chol


def get_nll(dtm, dom, means, cholcovs):
    """``filter.py:96-102`` (returns minus the summed log-likelihood)."""
    om_, oc_ = get_obs(*dtm, *dom, means[:-1], cholcovs[:-1])
    return -np.sum(mvn_loglikelihood(om_, oc_))


def get_sigma_squared(dtm, dom, means, cholcovs):
    """``filter.py:105-114``: sum ||whiten||^2 / (N-1) / d (whiten quirk)."""
    N, d = dom[1].shape
    om_, oc_ = get_obs(*dtm, *dom, means[:-1], cholcovs[:-1])
    ress = whiten(om_, oc_)
    return np.sum(ress * ress) / N / d


def sigma_squared_envelope(dtm, dom, means, cholcovs):
    """Range of the reference's sigma^2 (filter.py:105-114) over the column
    signs of the observation chols.

    ``whiten`` (utils.py:110-112) solves with L^T, so a step's term
    r^T (L^T L)^{-1} r changes when columns of L flip sign (L -> L S); every
    lower-triangular factor of the (full-rank) observation covariance is such
    an L S, and which one a QR returns is decided by rounding for
    rank-deficient filtered covariances.  Returns (lo, hi): sigma^2 with the
    smallest / largest term per step."""
    import itertools

    N, d = dom[1].shape
    om_, oc_ = get_obs(*dtm, *dom, means[:-1], cholcovs[:-1])
    G = np.linalg.inv(T(oc_) @ oc_)  # (L^T L)^{-1}
    signs = [np.array((1.0,) + s) for s in itertools.product((1.0, -1.0), repeat=d - 1)]
    vals = np.stack([np.einsum("ni,nij,nj->n", om_ * s, G, om_ * s) for s in signs])
    lo = vals.min(0).sum() / N / d
    hi = vals.max(0).sum() / N / d
    return lo, hi


def filter_objective(dtm, means):
    """``filter.py:43-45``: argument order swapped as in the reference."""
    F, QL = dtm
    return np.sum(objective_function_value(means[:-1], means[1:], F, QL))


def linear_noiseless_filtering(x0, dtm, dom, scan=associative_scan):
    """``filter.py:18-47``: returns ((means, chols), nll, obj, ssq)."""
    F, QL = dtm
    H, c, R = dom
    N = H.shape[0]
    ms = np.concatenate([x0[0][None], np.zeros((N - 1,) + x0[0].shape)])
    Ls = np.concatenate([x0[1][None], np.zeros((N - 1,) + x0[1].shape)])
    elems = get_element(F, QL, H, c, R, ms, Ls)
    _, means, cholcovs, _, _ = scan(sqrt_filtering_operator, elems)
    means = np.concatenate([x0[0][None], means])
    cholcovs = np.concatenate([x0[1][None], cholcovs])
    ssq = get_sigma_squared(dtm, dom, means, cholcovs)
    nll = get_nll(dtm, dom, means, cholcovs)
    obj = filter_objective(dtm, means)
    return (means, cholcovs), nll, obj, ssq


# --------------------------------------------------------------------------
# parallel smoother, pof/parallel_filtsmooth/smoother.py
# --------------------------------------------------------------------------


def sqrt_associative_params(F, cholQ, m, chol_P):
    """``smoother.py:37-50``: smoother element (g, E, D) of one step."""
    nx = cholQ.shape[-1]
    top = np.concatenate((F @ chol_P, cholQ), axis=-1)
    bot = np.concatenate((chol_P, np.zeros_like(cholQ)), axis=-1)
    TP = tria(np.concatenate((top, bot), axis=-2))
    Phi11 = TP[..., :nx, :nx]
    Phi21 = TP[..., nx:, :nx]
    D = TP[..., nx:, nx:]
    # general LU solve, as jlinalg.solve in the reference
    E = T(np.linalg.solve(T(Phi11), T(Phi21)))
    g = m - mv(E, mv(F, m))
    return g, E, D


def get_smoother_elements(dtm, filt):
    """``smoother.py:25-34``: N-1 elements plus the terminal (m_T, 0, L_T)."""
    F, QL = dtm
    ms, Ps = filt
    gs, Es, Ls = sqrt_associative_params(F, QL, ms[:-1], Ps[:-1])
    gs = np.concatenate([gs, ms[-1][None]])
    Es = np.concatenate([Es, np.zeros_like(Ps[-1])[None]])
    Ls = np.concatenate([Ls, Ps[-1][None]])
    return gs, Es, Ls


def sqrt_smoothing_operator(elem1, elem2):
    """``smoother.py:53-63``: elem1 is later in time, elem2 earlier."""
    g1, E1, D1 = elem1
    g2, E2, D2 = elem2
    g = mv(E2, g1) + g2
    E = E2 @ E1
    D = tria(np.concatenate([E2 @ D1, D2], axis=-1))
    return g, E, D


def smoothing(dtm, filt, scan=associative_scan):
    """``smoother.py:8-22``: returns ((means, chols), obj)."""
    elems = get_smoother_elements(dtm, filt)
    means, _, chols = scan(sqrt_smoothing_operator, elems, reverse=True)
    F, QL = dtm
    obj = np.sum(objective_function_value(means[:-1], means[1:], F, QL))
    return (means, chols), obj


def linear_filtsmooth(x0, dtm, dom, scan=associative_scan):
    """``pof/parallel_filtsmooth/__init__.py:5-10``: (states, nll(filter), obj(smoother), ssq)."""
    out, nll, _, ssq = linear_noiseless_filtering(x0, dtm, dom, scan=scan)
    out, obj = smoothing(dtm, out, scan=scan)
    return out, nll, obj, ssq


# --------------------------------------------------------------------------
# sequential twin, pof/sequential_filtsmooth/*
# --------------------------------------------------------------------------


def sqrt_predict(F, cholQ, m, cholP):
    """``sequential_filtsmooth/filter.py:59-66``."""
    return mv(F, m), tria(np.concatenate([F @ cholP, cholQ], axis=-1))


def sqrt_update(H, cholR, c, m, cholP):
    """``sequential_filtsmooth/filter.py:69-92``: returns (m, L), ell, ssq."""
    nx = m.shape[-1]
    ny = c.shape[-1]
    y_hat = mv(H, m) + c
    y_diff = 0 - y_hat
    top = np.concatenate([H @ cholP, cholR], axis=-1)
    bot = np.concatenate([cholP, np.zeros(cholP.shape[:-2] + (nx, ny))], axis=-1)
    chol_S = tria(np.concatenate([top, bot], axis=-2))
    cholP = chol_S[..., ny:, ny:]
    G = chol_S[..., ny:, :ny]
    I = chol_S[..., :ny, :ny]
    wres = whiten(y_diff, I)
    ssq = np.sum(wres * wres, -1) / ny
    m = m + mv(G, solve_tri(I, y_diff[..., None], lower=True)[..., 0])
    ell = mvn_loglikelihood(y_diff, I)
    return (m, cholP), ell, ssq


def linear_noiseless_filter(x0, dtm, dom):
    """``sequential_filtsmooth/filter.py:33-56``: returns (states, ell, ssq)."""
    F, QL = dtm
    H, c, R = dom
    n = F.shape[0]
    m, L = x0
    ms, Ls = [m], [L]
    ssq, ell = 0.0, 0.0
    for k in range(n):
        m, L = sqrt_predict(F[k], QL[k], m, L)
        (m, L), e, s = sqrt_update(H[k], R[k], c[k], m, L)
        ssq, ell = ssq + s, ell + e
        ms.append(m)
        Ls.append(L)
    return (np.stack(ms), np.stack(Ls)), ell, ssq / n


def extended_kalman_filter(x0, dtm, linearize):
    """``sequential_filtsmooth/filter.py:9-30``: linearizes at the predicted mean."""
    F, QL = dtm
    n = F.shape[0]
    m, L = x0
    ms, Ls = [m], [L]
    ssq, ell = 0.0, 0.0
    for k in range(n):
        m, L = sqrt_predict(F[k], QL[k], m, L)
        H, c, R = linearize(m)
        (m, L), e, s = sqrt_update(H, R, c, m, L)
        ssq, ell = ssq + s, ell + e
        ms.append(m)
        Ls.append(L)
    return (np.stack(ms), np.stack(Ls)), ell, ssq / n


def sqrt_smooth(F, cholQ, mf, Lf, ms, Ls):
    """``sequential_filtsmooth/smoother.py:31-48``."""
    nx = F.shape[-1]
    top = np.concatenate([F @ Lf, cholQ], axis=-1)
    bot = np.concatenate([Lf, np.zeros_like(F)], axis=-1)
    tp = tria(np.concatenate([top, bot], axis=-2))
    Phi11 = tp[..., :nx, :nx]
    Phi21 = tp[..., nx:, :nx]
    Phi22 = tp[..., nx:, nx:]
    gain = T(solve_tri(Phi11, T(Phi21), lower=True, trans=True))
    mean = mf + mv(gain, ms - mv(F, mf))
    chol = tria(np.concatenate([Phi22, gain @ Ls], axis=-1))
    return mean, chol


def sequential_smoothing(dtm, filt):
    """``sequential_filtsmooth/smoother.py:8-28``: returns (states, obj)."""
    F, QL = dtm
    fm, fL = filt
    n = F.shape[0]
    m, L = fm[-1], fL[-1]
    ms, Ls = [m], [L]
    for k in range(n - 1, -1, -1):
        m, L = sqrt_smooth(F[k], QL[k], fm[k], fL[k], m, L)
        ms.append(m)
        Ls.append(L)
    means = np.stack(ms[::-1])
    chols = np.stack(Ls[::-1])
    obj = np.sum(objective_function_value(means[:-1], means[1:], F, QL))
    return (means, chols), obj


def sequential_linear_filtsmooth(x0, dtm, dom):
    """``sequential_filtsmooth/__init__.py:13-16``: (states, ell (+), obj, ssq)."""
    out, nll, ssq = linear_noiseless_filter(x0, dtm, dom)
    out, obj = sequential_smoothing(dtm, out)
    return out, nll, obj, ssq


def sequential_filtsmooth(x0, dtm, linearize):
    """``sequential_filtsmooth/__init__.py:5-10`` (EKF + RTS)."""
    out, nll, ssq = extended_kalman_filter(x0, dtm, linearize)
    out, obj = sequential_smoothing(dtm, out)
    return out, nll, obj, ssq


__all__ = [
    "associative_scan",
    "sequential_scan",
    "get_element",
    "sqrt_filtering_operator",
    "linear_noiseless_filtering",
    "smoothing",
    "linear_filtsmooth",
    "sequential_linear_filtsmooth",
    "sequential_filtsmooth",
]
