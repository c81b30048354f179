"""The chunked three-phase parallel filter/smoother that the CUDA kernels
execute, restated in NumPy float64 (test infrastructure).

The reference computes the filtered and smoothed marginals with
``jax.lax.associative_scan`` over per-step elements
(``pof/parallel_filtsmooth/filter.py:18-47``, ``smoother.py:8-22``).  The
result of a scan does not depend on how the associative operator is
bracketed, so the CUDA path brackets it differently (same elements, same
operator, fewer flops), and this module restates that bracketing so the
kernels can be checked step by step:

Filter (steps s = 0..n-1, step s maps grid point s to s+1):
  phase 1, level 0 -- every chunk of C0 steps folds its elements into one
      element (A, b, U, eta, Z).  Instead of building each element
      (``filter.py:50-81``) and combining (``filter.py:117-142``), the fold
      runs the Kalman filter conditioned on the state at the chunk start:
      the mean stays affine in that state (A x + b), the gain does not depend
      on it, and the information the chunk's observations carry about it is
      accumulated as eta and Z Z^T.  Chunk 0 starts from x0 and yields the
      filtering state itself (A = 0, eta = 0, Z = 0).
  phase 2, levels >= 1 -- the chunk totals are folded the same way with the
      reference's operator ``sqrt_filtering_operator`` until few remain; one
      sequential pass gives the state at every top-level element start, and
      down-sweeps propagate states (b, U) through each chunk.
  phase 3, level 0 -- each chunk runs the square-root Kalman filter
      (``sequential_filtsmooth/filter.py:59-92``) from the state at its start,
      emitting the filtered marginals, the sigma^2 and NLL terms
      (``filter.py:84-114``: predicted observation from the filtered state at
      grid point s with the step-s model) and the filter objective terms.

Smoother (grid points k = 0..N-2; the state at N-1 is the filtered one):
  elements (g, E, D) as ``smoother.py:37-50``; chunks fold them forward with
  ``sqrt_smoothing_operator`` (``smoother.py:53-63``); the same hierarchy
  yields the smoothed state at every chunk end; each chunk then runs the
  backward recursion m_k = E_k m_{k+1} + g_k, L_k = tria([E_k L_{k+1}, D_k]).

All sums (sigma^2, NLL, objectives) are formed per chunk and then summed over
chunks in chunk order, the order the kernels use.
"""

import numpy as np

from .core import T, mvn_loglikelihood, solve_tri, tria, whiten
from .filtsmooth import mv, sqrt_filtering_operator, sqrt_smoothing_operator


def _chunks(n, C):
    return [(s, min(n, s + C)) for s in range(0, n, C)]


# --------------------------------------------------------------------------
# filter
# --------------------------------------------------------------------------


def kf_step(F, QL, H, c, R, m, L):
    """One square-root KF step (predict + noiseless update) from the filtered
    state (m, L) at grid s; returns the new state and the observation terms."""
    d = c.shape[-1]
    D = m.shape[-1]
    Lp = tria(np.concatenate([F @ L, QL], axis=-1))
    mp = mv(F, m)
    top = np.concatenate([H @ Lp, R], axis=-1)
    bot = np.concatenate([Lp, np.zeros(Lp.shape[:-2] + (D, d))], axis=-1)
    Psi = tria(np.concatenate([top, bot], axis=-2))
    P11 = Psi[..., :d, :d]
    P21 = Psi[..., d:, :d]
    U = Psi[..., d:, d:]
    r = mv(H, mp) + c  # predicted observation mean
    w = solve_tri(P11, (-r)[..., None], lower=True)[..., 0]
    m_new = mp + mv(P21, w)
    wq = whiten(r, P11)
    ssq_term = np.sum(wq * wq, -1)
    nll_term = -mvn_loglikelihood(r, P11)
    return m_new, U, ssq_term, nll_term, Lp


def conditional_fold(F, QL, H, c, R):
    """Fold the elements of one chunk (not containing x0) into (A, b, U, eta, Z)."""
    n, d, D = H.shape
    A = np.eye(D)
    b = np.zeros(D)
    L = np.zeros((D, D))
    eta = np.zeros(D)
    Z = np.zeros((D, D))
    for s in range(n):
        Fs = F[s]
        Lp = tria(np.concatenate([Fs @ L, QL[s]], axis=-1))
        top = np.concatenate([H[s] @ Lp, R[s]], axis=-1)
        bot = np.concatenate([Lp, np.zeros((D, d))], axis=-1)
        Psi = tria(np.concatenate([top, bot], axis=-2))
        P11, P21, U = Psi[:d, :d], Psi[d:, :d], Psi[d:, d:]
        FA = Fs @ A
        Fb = Fs @ b
        G = H[s] @ FA
        r = H[s] @ Fb + c[s]
        W = solve_tri(P11, G, lower=True)
        w = solve_tri(P11, r, lower=True)
        A = FA - P21 @ W
        b = Fb - P21 @ w
        eta = eta - W.T @ w
        Z = tria(np.concatenate([Z, W.T], axis=-1))
        L = U
    return A, b, L, eta, Z


def _fold_general(elems):
    """Left fold of general elements with the reference operator."""
    tot = tuple(e[0:1] for e in elems)
    for i in range(1, elems[0].shape[0]):
        tot = sqrt_filtering_operator(tot, tuple(e[i : i + 1] for e in elems))
    return tuple(t[0] for t in tot)


def _propagate_state(b1, U1, e2):
    """(b, U) part of ``sqrt_filtering_operator(e1, e2)`` (it reads only b1, U1 of e1)."""
    D = b1.shape[-1]
    e1 = (np.zeros((1, D, D)), b1[None], U1[None], np.zeros((1, D)), np.zeros((1, D, D)))
    out = sqrt_filtering_operator(e1, tuple(x[None] for x in e2))
    return out[1][0], out[2][0]


def _filter_states_ks(elems, m0, L0):
    """Filtering state before each element of a level by a Kogge-Stone
    prefix scan (the kernels' parallel top level, k_filt_ks_team): step s
    replaces P_i by P_{i-s} (x) P_i for i >= s; element 0 is absolute, so
    (b, U) of P_{i-1} is the state before element i."""
    n = elems[0].shape[0]
    P = [tuple(x[i : i + 1] for x in elems) for i in range(n)]
    s = 1
    while s < n:
        P = [P[i] if i < s else sqrt_filtering_operator(P[i - s], P[i]) for i in range(n)]
        s *= 2
    return [(m0, L0)] + [(P[i][1][0], P[i][2][0]) for i in range(n - 1)]


def _filter_states_at_starts(elems, Cs, m0, L0, ks_max=0):
    """Given level-l elements (element 0 holds x0), return the filtering state
    before each element: element 0 starts at x0; element i > 0 starts after
    elements 0..i-1.  Hierarchical with chunk sizes Cs; a level of at most
    ks_max (and more than 2) elements is scanned by _filter_states_ks."""
    n = elems[0].shape[0]
    C = Cs[0]
    if 2 < n <= ks_max:
        return _filter_states_ks(elems, m0, L0)
    if n <= C or len(Cs) == 1:
        states = [(m0, L0)]
        for i in range(n - 1):
            e = tuple(x[i] for x in elems)
            if i == 0:
                states.append((e[1], e[2]))
            else:
                states.append(_propagate_state(states[-1][0], states[-1][1], e))
        return states
    chunks = _chunks(n, C)
    totals = [_fold_general(tuple(x[s:t] for x in elems)) for s, t in chunks]
    totals = tuple(np.stack([tt[j] for tt in totals]) for j in range(5))
    starts = _filter_states_at_starts(totals, Cs[1:], m0, L0, ks_max)
    states = []
    for (s, t), st in zip(chunks, starts):
        cur = st
        states.append(cur)
        for i in range(s, t - 1):
            e = tuple(x[i] for x in elems)
            cur = (e[1], e[2]) if i == 0 else _propagate_state(cur[0], cur[1], e)
            states.append(cur)
    return states


def _filter_states_segmented(elems, Cg, m0, L0):
    """States before each element for the batched schedule: groups of Cg
    elements fold until one element remains, whose start state is x0; the
    down-sweep propagates through every group (no element is special)."""
    n = elems[0].shape[0]
    if n == 1:
        return [(m0, L0)]
    chunks = _chunks(n, Cg)
    totals = [_fold_general(tuple(x[s:t] for x in elems)) for s, t in chunks]
    totals = tuple(np.stack([tt[j] for tt in totals]) for j in range(5))
    starts = _filter_states_segmented(totals, Cg, m0, L0)
    states = []
    for (s, t), st in zip(chunks, starts):
        cur = st
        states.append(cur)
        for i in range(s, t - 1):
            cur = _propagate_state(cur[0], cur[1], tuple(x[i] for x in elems))
            states.append(cur)
    return states


def filter_blocked(x0, dtm, dom, C0=4, Cs=(4,), segmented=False, ks_max=0):
    """Filtered marginals with the chunked schedule; returns
    ((means, chols), nll, obj, ssq, chunk_states).  ks_max: the largest level
    scanned by a parallel prefix scan instead of the tree (0: none).

    segmented=True restates the batched solve's schedule for one problem
    (csrc/pof_batch.cuh): chunk 0 is a conditional fold like the others, the
    levels above fold groups of Cs[0] until one element remains, and x0 is
    the state before it."""
    F, QL = dtm
    H, c, R = dom
    n, d, D = H.shape
    m0, L0 = x0
    chunks = _chunks(n, C0)
    # phase 1: chunk totals
    totals = []
    for j, (s, t) in enumerate(chunks):
        if j == 0 and not segmented:
            m, L = m0, L0
            for k in range(s, t):
                m, L, _, _, _ = kf_step(F[k], QL[k], H[k], c[k], R[k], m, L)
            totals.append((np.zeros((D, D)), m, L, np.zeros(D), np.zeros((D, D))))
        else:
            totals.append(conditional_fold(F[s:t], QL[s:t], H[s:t], c[s:t], R[s:t]))
    totals = tuple(np.stack([tt[j] for tt in totals]) for j in range(5))
    # phase 2: state at every chunk start
    if segmented:
        starts = _filter_states_segmented(totals, Cs[0], m0, L0)
    else:
        starts = _filter_states_at_starts(totals, list(Cs), m0, L0, ks_max)
    # phase 3: KF inside every chunk
    means = [m0]
    chols = [L0]
    ssq_c, nll_c, obj_c = [], [], []
    for (s, t), (m, L) in zip(chunks, starts):
        ss = nn = oo = 0.0
        for k in range(s, t):
            m_new, L_new, st, nt, _ = kf_step(F[k], QL[k], H[k], c[k], R[k], m, L)
            ss += st
            nn += nt
            r = solve_tri(QL[k], m - F[k] @ m_new, lower=True)
            oo += r @ r
            means.append(m_new)
            chols.append(L_new)
            m, L = m_new, L_new
        ssq_c.append(ss)
        nll_c.append(nn)
        obj_c.append(oo)
    ssq = sum(ssq_c) / n / d
    nll = sum(nll_c)
    obj = sum(obj_c)
    return (np.stack(means), np.stack(chols)), nll, obj, ssq, starts


# --------------------------------------------------------------------------
# smoother
# --------------------------------------------------------------------------


def smoother_element(F, QL, m, L):
    """``smoother.py:37-50`` with a triangular solve for E (Phi11 is triangular)."""
    D = m.shape[-1]
    top = np.concatenate([F @ L, QL], axis=-1)
    bot = np.concatenate([L, np.zeros((D, D))], axis=-1)
    Phi = tria(np.concatenate([top, bot], axis=-2))
    P11, P21, P22 = Phi[:D, :D], Phi[D:, :D], Phi[D:, D:]
    E = solve_tri(P11, P21.T, lower=True, trans=True).T
    g = m - E @ (F @ m)
    return g, E, P22


def _fold_smoother(elems):
    """Composite of smoother elements in time order: maps the smoothed state
    after the chunk to the smoothed state at its first grid point."""
    tot = tuple(e[0:1] for e in elems)
    for i in range(1, elems[0].shape[0]):
        tot = sqrt_smoothing_operator(tuple(e[i : i + 1] for e in elems), tot)
    return tuple(t[0] for t in tot)


def _apply_composite(e, m, L):
    g, E, D = e
    return E @ m + g, tria(np.concatenate([E @ L, D], axis=-1))


def _smoother_ends_ks(elems, mT, LT):
    """Smoothed state after each element of a level by a Kogge-Stone suffix
    scan (k_smo_abs_team, k_smo_ks_team): the terminal state is pushed
    through the last element, which becomes absolute (E = 0); step s
    replaces S_i by S_i o S_{i+s} for i + s < n; (g, D) of S_i is then the
    state at the start of element i, i.e. after element i - 1."""
    n = elems[0].shape[0]
    S = [tuple(x[i : i + 1] for x in elems) for i in range(n)]
    g, L = _apply_composite(tuple(x[0] for x in S[-1]), mT, LT)
    D = g.shape[-1]
    S[-1] = (g[None], np.zeros((1, D, D)), L[None])
    s = 1
    while s < n:
        S = [sqrt_smoothing_operator(S[i + s], S[i]) if i + s < n else S[i] for i in range(n)]
        s *= 2
    return [(S[i][0][0], S[i][2][0]) for i in range(1, n)] + [(mT, LT)]


def _smoother_states_at_ends(elems, Cs, mT, LT, ks_max=0):
    """Smoothed state right after each element (element i maps the state at
    its end to the state at its start); the last element ends at the terminal.
    A level of at most ks_max (and more than 2) elements is scanned by
    _smoother_ends_ks."""
    n = elems[0].shape[0]
    C = Cs[0]
    if 2 < n <= ks_max:
        return _smoother_ends_ks(elems, mT, LT)
    if n <= C or len(Cs) == 1:
        ends = [None] * n
        cur = (mT, LT)
        for i in range(n - 1, -1, -1):
            ends[i] = cur
            cur = _apply_composite(tuple(x[i] for x in elems), *cur)
        return ends
    chunks = _chunks(n, C)
    totals = [_fold_smoother(tuple(x[s:t] for x in elems)) for s, t in chunks]
    totals = tuple(np.stack([tt[j] for tt in totals]) for j in range(3))
    cends = _smoother_states_at_ends(totals, Cs[1:], mT, LT, ks_max)
    ends = [None] * n
    for (s, t), ce in zip(chunks, cends):
        cur = ce
        for i in range(t - 1, s - 1, -1):
            ends[i] = cur
            cur = _apply_composite(tuple(x[i] for x in elems), *cur)
    return ends


def _smoother_states_segmented(elems, Cg, mT, LT):
    """Smoothed state after each element for the batched schedule: groups of
    Cg fold until one element remains, which ends at the terminal state."""
    n = elems[0].shape[0]
    if n == 1:
        return [(mT, LT)]
    chunks = _chunks(n, Cg)
    totals = [_fold_smoother(tuple(x[s:t] for x in elems)) for s, t in chunks]
    totals = tuple(np.stack([tt[j] for tt in totals]) for j in range(3))
    cends = _smoother_states_segmented(totals, Cg, mT, LT)
    ends = [None] * n
    for (s, t), ce in zip(chunks, cends):
        cur = ce
        for i in range(t - 1, s - 1, -1):
            ends[i] = cur
            cur = _apply_composite(tuple(x[i] for x in elems), *cur)
    return ends


def smoother_blocked(dtm, filt, C0=4, Cs=(4,), segmented=False, ks_max=0):
    """Smoothed marginals with the chunked schedule; returns ((means, chols), obj).
    segmented=True: the batched solve's hierarchy (see filter_blocked); ks_max
    as in filter_blocked."""
    F, QL = dtm
    fm, fL = filt
    N, D = fm.shape
    n = N - 1
    g = np.zeros((n, D))
    E = np.zeros((n, D, D))
    Dk = np.zeros((n, D, D))
    for k in range(n):
        g[k], E[k], Dk[k] = smoother_element(F[k], QL[k], fm[k], fL[k])
    chunks = _chunks(n, C0)
    totals = [_fold_smoother((g[s:t], E[s:t], Dk[s:t])) for s, t in chunks]
    totals = tuple(np.stack([tt[j] for tt in totals]) for j in range(3))
    if segmented:
        ends = _smoother_states_segmented(totals, Cs[0], fm[-1], fL[-1])
    else:
        ends = _smoother_states_at_ends(totals, list(Cs), fm[-1], fL[-1], ks_max)
    means = np.zeros((N, D))
    chols = np.zeros((N, D, D))
    means[-1], chols[-1] = fm[-1], fL[-1]
    obj_c = []
    for (s, t), (m, L) in zip(chunks, ends):
        oo = 0.0
        for k in range(t - 1, s - 1, -1):
            m_new, L_new = _apply_composite((g[k], E[k], Dk[k]), m, L)
            r = solve_tri(QL[k], m_new - F[k] @ m, lower=True)
            oo += r @ r
            means[k], chols[k] = m_new, L_new
            m, L = m_new, L_new
        obj_c.append(oo)
    return (means, chols), sum(obj_c)


def linear_filtsmooth_blocked(x0, dtm, dom, C0=4, Cs=(4,), segmented=False, ks_max=0):
    """``pof/parallel_filtsmooth/__init__.py:5-10`` with the chunked schedule."""
    out, nll, _, ssq, _ = filter_blocked(x0, dtm, dom, C0=C0, Cs=Cs, segmented=segmented, ks_max=ks_max)
    out, obj = smoother_blocked(dtm, out, C0=C0, Cs=Cs, segmented=segmented, ks_max=ks_max)
    return out, nll, obj, ssq


def segmented_filtsmooth(C0, Cg):
    """linear_filtsmooth with the batched solve's schedule, for
    oracle.solver.solve(..., filtsmooth=...)."""

    def fs(x0, dtm, dom):
        return linear_filtsmooth_blocked(x0, dtm, dom, C0=C0, Cs=(Cg,), segmented=True)

    return fs
