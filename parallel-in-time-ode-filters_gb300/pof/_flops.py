"""Floating-point operation counts of libpof's kernels (host-side model).

Counts follow the loops of csrc/pof_linalg.cuh and csrc/pof_ops.cuh one to
one: an FMA is 2 flops; add, multiply, divide, square root and log are 1.
They are the algorithmic work of each kernel, the numerator of its
achieved-FLOP/s figure.  ``reference_step_flops`` is the work per step and
IEKS iteration of the reference's own formulation (per-step elements,
~2 combines per element in the associative scan, sigma^2/NLL pass).
"""


def tria(M, NC, MB=0):
    """tria<M, NC> (+ MB extra rows for tria_top)."""
    f = 0
    for j in range(M):
        t = NC - j - 1
        f += 2 * t + 2 + 1 + 3 + t  # |x|^2, nrm (fma + sqrt), beta/tau/scal, scale tail
        rows = (M - j - 1) + MB
        f += rows * (4 * t + 2)
    return f


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


def kf_step(D, d, smooth):
    f = mm_lowerB(D, D)
    if smooth:
        f += tria(D, 2 * D, MB=D) + tria(D, D)
        f += trsm(D, D) + mv(D, D) + D
    else:
        f += tria(D, 2 * D)
    f += mv(D, D)  # predicted mean
    f += mm_lowerB(d, D)  # H Lp (Lp lower)
    f += tria(D + d, D + d)
    f += mv(d, D) + d  # r
    f += 2 * trsv(d)
    f += d * (2 + 2 + 1)  # ssq, y^2, log
    f += 5
    f += D * 2 * d  # mean update
    return f


def cond_fold_step(D, d):
    f = mm_lowerB(D, D) + tria(D, 2 * D)
    f += mm_lowerB(d, D) + tria(D + d, D + d)
    f += mm(D, D, D) + mv(D, D)  # F A, F b
    f += mm(d, D, D) + mv(d, D) + d  # H FA, H Fb + c
    f += trsm(d, D) + trsv(d)
    f += D * D * 2 * d + D * 2 * d + D * 2 * d  # A, b, eta
    f += tria(D, D + d)
    return f


def filt_combine(D):
    f = mm(D, D, D)  # U1^T Z2
    f += tria(D, 2 * D, MB=D) + tria(D, D)
    f += mm(D, D, D) + trsm(D, D)  # M
    f += trsm(D, D)  # Mu
    f += mm(D, D, D)  # MX
    f += mm(D, D, D) + D * D  # A
    f += 2 * mv(D, D) + D + mv(D, D) + mv(D, D) + D + mv(D, D) + D  # b
    f += trsm(D, D)  # e
    f += 2 * mv(D, D) + D + mv(D, D) + mv(D, D) + D + mv(D, D) + D  # eta
    f += tria(D, 2 * D)  # U
    f += mm(D, D, D) + tria(D, 2 * D)  # Z
    return f


def filt_apply(D):
    f = mm(D, D, D) + tria(D, 2 * D, MB=D)
    f += mm(D, D, D) + trsm(D, D) + trsm(D, D)
    f += 2 * mv(D, D) + D + mv(D, D) + mv(D, D) + D + mv(D, D) + D
    f += tria(D, 2 * D)
    return f


def smooth_combine(D):
    return mv(D, D) + mm_lowerB(D, D) + tria(D, 2 * D) + mm(D, D, D) + D


def smooth_apply(D):
    return mv(D, D) + mm_lowerB(D, D) + tria(D, 2 * D) + D


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
        return (n - n1) * smooth_combine(D)
    if kind == "smo_l0_down":
        return n * (smooth_apply(D) + objective_term(D) + D * D)
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
