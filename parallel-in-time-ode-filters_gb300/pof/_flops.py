"""Floating-point operation counts of libpof's kernels (host-side model).

Counts follow the loops of the kernels: an FMA is 2 flops; add, multiply,
divide, square root and log are 1.  They are the algorithmic work of each
kernel -- the operations it performs, the structural zeros it skips not
counted (a few products over a triangular factor that the team kernels run
dense are counted at their triangular size, mm_lowerB, so the figure errs
low) -- and the numerator of its achieved-FLOP/s figure.  The thread-per-
chunk level 0 (D < 6, csrc/pof_ops.cuh) runs the dense loops; the team
kernels (level 0 from D = 6 on, every level >= 1, csrc/pof_team.cuh) skip the
zeros of the lower-triangular right blocks of the triangularizations, the
zero columns of the noiseless update and the zero blocks of the IWP
transition matrix (structured=True).  ``reference_step_flops`` is the work
per step and IEKS iteration of the reference's own formulation (per-step
elements, ~2 combines per element in the associative scan, sigma^2/NLL pass).
"""


def tria(M, NC, MB=0, wlow=0, ncut=None):
    """tria<M, NC> (+ MB extra rows for tria_top); wlow > 0: the right block
    from column wlow is lower-triangular, reflector j stops at column
    wlow + j; ncut: the columns from ncut on are zero (reflectors from
    ncut - 1 on are skipped)."""
    f = 0
    mlim = M if ncut is None else min(M, ncut - 1)
    for j in range(mlim):
        kend = NC if wlow <= 0 else min(NC, wlow + j + 1)
        if ncut is not None:
            kend = min(kend, ncut)
        t = kend - j - 1
        f += 2 * t + 2 + 1 + 3 + t  # |x|^2, nrm (fma + sqrt), beta/tau/scal, scale tail
        rows = (M - j - 1) + MB
        f += rows * (4 * t + 2)
    return f


def mm_f(D, N, d):
    """F B for the IWP transition matrix F = I_d (x) A_1, A_1 upper-triangular
    (q + 1) x (q + 1): row i of F has (q + 1) - i mod (q + 1) nonzeros."""
    Q = D // d
    return 2 * N * d * (Q * (Q + 1) // 2)


def mm(M, K, N):
    return 2 * M * K * N


def mm_lowerB(M, K):
    return 2 * M * K * (K + 1) // 2


def mv(M, N):
    return 2 * M * N


def trsv(M):
    return M * (M - 1) + M


def trsm(M, NR):
    return NR * M * (M - 1) + M * NR + M


def kf_step(D, d, smooth, structured=None):
    st = D >= 6 if structured is None else structured
    w = D if st else 0
    f = mm_f(D, D, d) if st else mm_lowerB(D, D)
    if smooth:
        f += tria(D, 2 * D, MB=D, wlow=w) + tria(D, D)
        f += trsm(D, D) + mv(D, D) + D
    else:
        f += tria(D, 2 * D, wlow=w)
    f += mm_f(D, 1, d) if st else mv(D, D)  # predicted mean
    f += mm_lowerB(d, D)  # H Lp (Lp lower)
    f += tria(D + d, D + d, ncut=D if st else None)
    f += mv(d, D) + d  # r
    f += 2 * trsv(d)
    f += d * (2 + 2 + 1)  # ssq, y^2, log
    f += 5
    f += D * 2 * d  # mean update
    return f


def cond_fold_step(D, d, structured=None):
    st = D >= 6 if structured is None else structured
    f = (mm_f(D, D, d) + tria(D, 2 * D, wlow=D)) if st else (mm_lowerB(D, D) + tria(D, 2 * D))
    f += mm_lowerB(d, D) + tria(D + d, D + d, ncut=D if st else None)
    f += (mm_f(D, D, d) + mm_f(D, 1, d)) if st else (mm(D, D, D) + mv(D, D))  # F A, F b
    f += mm(d, D, D) + mv(d, D) + d  # H FA, H Fb + c
    f += trsm(d, D) + trsv(d)
    f += D * D * 2 * d + D * 2 * d + D * 2 * d  # A, b, eta
    f += tria(D, D + d)
    return f


def filt_combine(D):
    f = mm(D, D, D)  # U1^T Z2
    f += tria(D, 2 * D, MB=D, wlow=D) + tria(D, D)
    f += mm(D, D, D) + trsm(D, D)  # M
    f += trsm(D, D)  # Mu
    f += mm(D, D, D)  # MX
    f += mm(D, D, D) + D * D  # A
    f += 2 * mv(D, D) + D + mv(D, D) + mv(D, D) + D + mv(D, D) + D  # b
    f += trsm(D, D)  # e
    f += 2 * mv(D, D) + D + mv(D, D) + mv(D, D) + D + mv(D, D) + D  # eta
    f += tria(D, 2 * D, wlow=D)  # U
    f += mm(D, D, D) + tria(D, 2 * D, wlow=D)  # Z
    return f


def filt_apply(D):
    f = mm(D, D, D) + tria(D, 2 * D, MB=D, wlow=D)
    f += mm(D, D, D) + trsm(D, D) + trsm(D, D)
    f += 2 * mv(D, D) + D + mv(D, D) + mv(D, D) + D + mv(D, D) + D
    f += tria(D, 2 * D, wlow=D)
    return f


def smooth_combine(D, structured=True):
    w = D if structured else 0
    return mv(D, D) + mm_lowerB(D, D) + tria(D, 2 * D, wlow=w) + mm(D, D, D) + D


def smooth_apply(D, structured=True):
    w = D if structured else 0
    return mv(D, D) + mm_lowerB(D, D) + tria(D, 2 * D, wlow=w) + D


def objective_term(D):
    return mv(D, D) + D + trsv(D) + 2 * D


def kernel_flops(kind, n, D, d, C0, cnt):
    """Flops of one launch of a kernel kind over a problem with n steps and
    level sizes cnt = [None, cnt1, cnt2, ...] (all launches of that kind in
    one filter + smoother pass, summed over levels)."""
    n1 = cnt[1]
    levels = len(cnt) - 1
    if kind == "filt_l0_reduce":
        first = min(C0, n)
        return first * kf_step(D, d, False) + (n - first) * cond_fold_step(D, d)
    if kind == "filt_l0_down":
        return n * (kf_step(D, d, True) + objective_term(D))
    if kind == "smo_l0_reduce":
        return (n - n1) * smooth_combine(D, D >= 6)
    if kind == "smo_l0_down":
        return n * (smooth_apply(D, D >= 6) + objective_term(D) + D * D)
    if kind == "filt_reduce":
        return sum(cnt[l] - cnt[l + 1] for l in range(1, levels)) * filt_combine(D)
    if kind == "filt_down":
        return sum(cnt[l] - cnt[l + 1] for l in range(1, levels)) * filt_apply(D)
    if kind == "smo_reduce":
        return sum(cnt[l] - cnt[l + 1] for l in range(1, levels)) * smooth_combine(D)
    if kind == "smo_down":
        return sum(cnt[l] - cnt[l + 1] for l in range(1, levels)) * smooth_apply(D)
    if kind == "filt_top":
        return max(cnt[levels] - 1, 0) * filt_apply(D)
    if kind == "smo_top":
        return max(cnt[levels] - 1, 0) * smooth_apply(D)
    return 0


def l0_lanes(D):
    """Lanes per level-0 chunk (csrc/pof_plan.h: narrow teams from D = 6 on)."""
    if D < 6:
        return 1
    wide = 8 if 2 * D <= 8 else (16 if 2 * D <= 16 else 32)
    return max(wide // 2, 4)


def plan_levels(n, D=4, C0=None, Cg=2, top=2):
    """The level sizes libpof uses (csrc/pof_plan.h make_plan)."""
    if C0 is None:
        lanes = l0_lanes(D)
        C0 = 4 if lanes == 1 else 2
        target = 16384 if lanes == 1 else max(1024, 65536 // lanes)
        while C0 < 64 and n // C0 > target:
            C0 *= 2
    cnt = [None, (n + C0 - 1) // C0]
    while cnt[-1] > top:
        cnt.append((cnt[-1] + Cg - 1) // Cg)
    return C0, cnt


def iteration_flops(n, D, d):
    """All kernels of one IEKS iteration (filter + smoother), by kind."""
    C0, cnt = plan_levels(n, D)
    kinds = ["filt_l0_reduce", "filt_reduce", "filt_top", "filt_down", "filt_l0_down", "smo_l0_reduce",
             "smo_reduce", "smo_top", "smo_down", "smo_l0_down"]
    return {k: kernel_flops(k, n, D, d, C0, cnt) for k in kinds}


def reference_step_flops(D, d):
    """Per step and IEKS iteration in the reference's formulation: element,
    ~2 filter combines, smoother element, ~2 smoother combines, observation
    pass (as in pof/parallel_filtsmooth/filter.py and smoother.py)."""
    def tr(m, nn):
        return 2 * m * m * nn - 2 * m ** 3 / 3

    Ef = 16 / 3 * D ** 3 + 4 / 3 * (D + d) ** 3 + 6 * d * D ** 2 + 3 * d * d * D
    Cf = 91 / 3 * D ** 3 + 14 * D ** 2
    Es = 46 / 3 * D ** 3 + 4 * D ** 2
    Cs = 22 / 3 * D ** 3 + 2 * D ** 2
    O = 16 / 3 * D ** 3 + 2 * d * D ** 2 + tr(d, D + d) + 4 * D ** 2
    return Ef + 2 * Cf + Es + 2 * Cs + O


def kernel_bytes(n, D, d, esz=8):
    """Compulsory DRAM bytes of one launch of the level-0 kernels over a
    problem of n steps (each input read once, each output written once, in
    the workspace layout of csrc/pof_plan.h): the `algorithmic` traffic the
    roofline compares ncu's dram bytes with."""
    C0, cnt = plan_levels(n, D)
    n1 = cnt[1]
    elem = 3 * D * D + 2 * D  # filter element (A, b, U, eta, Z)
    state = D + D * D  # (mean, chol)
    selem = D + 2 * D * D  # smoother element (g, E, D)
    return {
        "linearize": esz * n * (D + d * D + d),
        "filt_l0_reduce": esz * (n * (d * D + d) + n1 * elem),
        # H, c in; chunk start states in; means, chols, smoother elements out
        "filt_l0_down": esz * (n * (d * D + d + state + selem) + n1 * state),
        "smo_l0_reduce": esz * (n * selem + n1 * selem),
        # smoother elements, previous means in; chunk end states in; means, chols out
        "smo_l0_down": esz * (n * (selem + D + state) + n1 * state),
    }


# ---------------------------------------------------------------------------
# the dense path (csrc/pof_dense_sched.h): flops as its launches run them,
# GEMM M N K -> 2 M N K, tria of an m x n block -> 2 m^2 n - 2/3 m^3 (the
# Householder LQ's arithmetic, without the compact-WY overhead), triangular
# solve M x K -> M^2 K.  Per step and filter + smoother pass; the top levels
# (P - 1 sequential combines each way) are added per chunk.
# ---------------------------------------------------------------------------


def _tri(m, n):
    return 2.0 * m * m * n - 2.0 * m ** 3 / 3.0


def dense_step_flops(D, d):
    """Flops per step of one dense filter + smoother pass (phases 1 and 3 of
    the filter, the smoother's elements, chunk composites and backward
    recursion)."""
    g = lambda m, n, k: 2.0 * m * n * k  # noqa: E731
    fold = (g(D, D, D) + _tri(D, 2 * D) + g(d, D, D) + _tri(d + D, D + d) + g(D, D + 1, D) + g(d, D + 1, D)
            + d * d * (D + 1) + g(D, D + 1, d) + g(D, 1, d) + _tri(D, D + d))
    kf = g(D, D, D) + _tri(D, 2 * D) + g(D, 1, D) + g(d, D, D) + _tri(d + D, D + d) + g(d, 1, D) + 2 * d * d + g(D, 1, d)
    elem = g(D, D, D) + _tri(2 * D, 2 * D) + D ** 3 + g(D, 1, D) * 2
    comp = 2 * g(D, D, D) + g(D, 1, D) + _tri(D, 2 * D)
    back = g(D, 1, D) + g(D, D, D) + _tri(D, 2 * D)
    objectives = 2 * (g(D, 1, D) + D * D)
    return fold + kf + elem + comp + back + objectives


def dense_top_flops(D, d):
    """Flops of one chunk boundary of the top levels (a filter propagate and
    a smoother application)."""
    g = lambda m, n, k: 2.0 * m * n * k  # noqa: E731
    prop = g(D, D, D) + _tri(2 * D, 2 * D) + D ** 3 + 6 * g(D, 1, D) + g(D, D, D) + _tri(D, 2 * D)
    app = g(D, 1, D) + g(D, D, D) + _tri(D, 2 * D)
    return prop + app


def dense_pass_flops(n, D, d, chunks):
    """Flops of one dense filter + smoother pass over n steps with `chunks` chunks."""
    return n * dense_step_flops(D, d) + max(chunks - 1, 0) * dense_top_flops(D, d)
