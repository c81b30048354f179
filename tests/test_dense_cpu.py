"""The dense (large-D) filter/smoother schedule of libpof
(csrc/pof_dense_sched.h) on the host, no GPU: the schedule's host code runs
with plain-loop primitives that check every element access against the
workspace, inputs and outputs (tests/dense_sched_cpu.cpp; the workspace
starts as NaN, so a read of scratch nothing wrote poisons the results).  Its
outputs equal the oracle's segmented chunked schedule
(oracle.blocked.linear_filtsmooth_blocked(segmented=True)) with the same
chunks to rounding, and the reference scan (oracle.filtsmooth) to 1e-10:
filtered and smoothed means, covariances as L L^T, NLL, both objectives,
sigma^2 for d = 1; also the filter alone and the smoother alone, constant and
per-step transition models, zero and non-zero cholR, ragged last chunks."""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import blocked, filtsmooth as ofs, ivp as oivp, solver as osolver

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "parallel-in-time-ode-filters_gb300", "csrc")


@pytest.fixture(scope="module")
def dense_cpu(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    so = str(tmp_path_factory.mktemp("dense") / "dense_sched_cpu.so")
    src = os.path.join(ROOT, "tests", "dense_sched_cpu.cpp")
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-shared", "-fPIC", "-I", CSRC, src, "-o", so],
                   check=True, capture_output=True, text=True)
    lib = ctypes.CDLL(so)
    dp = ctypes.POINTER(ctypes.c_double)
    i32, i64 = ctypes.c_int32, ctypes.c_int64
    lib.dense_cpu_filtsmooth.argtypes = [i32, i64, i32, i32, dp, dp, dp, dp, i64, dp, dp, dp, i64, dp, dp, dp, i32,
                                         ctypes.c_char_p, i32]
    lib.dense_cpu_filtsmooth.restype = ctypes.c_int
    lib.dense_cpu_workspace_check.argtypes = [i32, i64, i32, i32, i32, ctypes.POINTER(ctypes.c_int64)]
    return lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _plan(lib, which, n, D, d, chunks):
    out = (ctypes.c_int64 * 5)()
    lib.dense_cpu_workspace_check(which, n, D, d, chunks, out)
    return {"total": out[0], "P": out[1], "C0": out[2], "last": out[3], "S": out[4]}


def _run(lib, which, x0m, x0L, F, QL, fts, H, c, R, rst, chunks, n, D, d):
    om = np.zeros((n + 1, D))
    oL = np.zeros((n + 1, D, D))
    osc = np.zeros(8)
    msg = ctypes.create_string_buffer(256)
    args = [np.ascontiguousarray(a) if a is not None else None for a in (x0m, x0L, F, QL, H, c, R)]
    rc = lib.dense_cpu_filtsmooth(which, n, D, d, _p(args[0]), _p(args[1]), _p(args[2]), _p(args[3]), fts,
                                  _p(args[4]), _p(args[5]), _p(args[6]), rst, _p(om), _p(oL), _p(osc), chunks, msg,
                                  256)
    assert rc == 0, msg.value.decode()
    return om, oL, osc


def _covd(a, b):
    A = a @ np.swapaxes(a, -1, -2)
    B = b @ np.swapaxes(b, -1, -2)
    return np.abs(A - B).max() / max(np.abs(B).max(), 1e-300)


def _converged_problem(ivp, N, q, iters):
    ts = np.linspace(ivp.t0, ivp.tmax, N)
    states, info, st = osolver.solve(ivp, ts, q, init="constant", maxiters=iters, return_full=True)
    dom = osolver.linearize_at_previous_states(st, states[0])
    return st, (st.F, st.QL), dom


def _random_problem(rng, n, D, d, with_R):
    """A well-conditioned linear model with per-step transitions near the
    identity and noisy or noiseless observations of d mixtures of the state."""
    F = np.eye(D) + 0.05 * rng.standard_normal((n, D, D))
    QL = np.tril(0.1 * rng.standard_normal((n, D, D)))
    QL[:, np.arange(D), np.arange(D)] = 0.2 + 0.1 * rng.random((n, D))
    H = rng.standard_normal((n, d, D))
    c = rng.standard_normal((n, d))
    R = None
    if with_R:
        R = np.tril(0.1 * rng.standard_normal((n, d, d)))
        R[:, np.arange(d), np.arange(d)] = 0.3
    m0 = rng.standard_normal(D)
    L0 = np.tril(0.2 * rng.standard_normal((D, D))) + 0.5 * np.eye(D)
    return (m0, L0), (F, QL), (H, c, R)


def _expected(x0, dtm, dom, C0, P):
    F, QL = dtm
    H, c, R = dom
    n, d, D = H.shape
    Rs = np.zeros((n, d, d)) if R is None else R
    dom_o = (H, c, Rs)
    (fm, fL), nll, fobj, ssq, _ = blocked.filter_blocked(x0, (F, QL), dom_o, C0=C0, Cs=(2,), segmented=True)
    (sm, sL), sobj = blocked.smoother_blocked((F, QL), (fm, fL), C0=C0, Cs=(2,), segmented=True)
    return (fm, fL), (sm, sL), nll, fobj, sobj, ssq


def _check(got, want, tol, what):
    err = np.abs(got - want).max() / max(np.abs(want).max(), 1e-300)
    assert err <= tol, "%s: %.3e > %.0e" % (what, err, tol)


CASES = [
    ("logistic_q2", lambda: _converged_problem(oivp.logistic(r=3.0), 41, 2, 30)),
    ("vdp_q3", lambda: _converged_problem(oivp.vanderpol(stiffness_constant=1.0), 37, 3, 30)),
    ("rigid_q3", lambda: _converged_problem(oivp.rigid_body(), 29, 3, 20)),
]


@pytest.mark.parametrize("chunks", [1, 4, 7, 0])
@pytest.mark.parametrize("name,mk", CASES)
def test_dense_schedule_matches_oracle_on_solver_models(dense_cpu, name, mk, chunks):
    st, dtm, dom = mk()
    H, c, R = dom
    n, d, D = H.shape
    F, QL = dtm
    pl = _plan(dense_cpu, 1, n, D, d, chunks)
    m0, L0 = st.x0
    om, oL, osc = _run(dense_cpu, 1, m0, L0, F[0], QL[0], 0, H, c, None, 0, chunks, n, D, d)
    (fm, fL), (sm, sL), nll, fobj, sobj, ssq = _expected(st.x0, dtm, dom, pl["C0"], pl["P"])
    _check(om, sm, 1e-11, "smoothed means")
    assert _covd(oL, sL) <= 1e-11
    _check(osc[0], nll, 1e-11, "nll")
    _check(osc[1], sobj, 1e-10, "smoother objective")
    _check(osc[3], fobj, 1e-10, "filter objective")
    if d == 1:
        _check(osc[2], ssq, 1e-11, "sigma^2")
    # and the reference scan, to the blocked/reference spread
    (rm, rL), rnll, robj, rssq = ofs.linear_filtsmooth(st.x0, dtm, dom)
    _check(om, rm, 1e-10, "smoothed means vs the reference scan")
    assert _covd(oL, rL) <= 1e-10


@pytest.mark.parametrize("n,D,d,chunks,with_R,per_step", [
    (23, 20, 3, 5, True, True),
    (16, 33, 4, 4, False, True),
    (9, 24, 24, 3, True, False),
    (1, 18, 2, 0, False, True),
    (12, 12, 5, 12, True, True),
    (23, 20, 3, 4, False, True),   # C0 = 6, last chunk 5 steps (odd shortfall)
    (33, 16, 2, 4, True, False),   # C0 = 9, last chunk 6 steps
    (29, 10, 2, 8, False, True),   # C0 = 4, last chunk 1 step
    (23, 14, 1, 4, True, True),    # d = 1: sigma^2 compared
    (300, 10, 2, 256, False, True),  # C0 = 2, 150 chunks: tree levels 150, 75, 38, 19, 10, 5, 3, 2, 1
    (97, 12, 3, 33, True, False),    # C0 = 3, 33 chunks (odd levels all the way up)
])
def test_dense_schedule_matches_oracle_on_random_models(dense_cpu, n, D, d, chunks, with_R, per_step):
    rng = np.random.default_rng(n * 1000 + D * 10 + d)
    x0, dtm, dom = _random_problem(rng, n, D, d, with_R)
    F, QL = dtm
    if not per_step:
        F = np.broadcast_to(F[0], F.shape).copy()
        QL = np.broadcast_to(QL[0], QL.shape).copy()
        dtm = (F, QL)
    H, c, R = dom
    pl = _plan(dense_cpu, 1, n, D, d, chunks)
    fts = D * D if per_step else 0
    rst = d * d if R is not None else 0
    Fa, QLa = (F, QL) if per_step else (F[0], QL[0])
    om, oL, osc = _run(dense_cpu, 1, x0[0], x0[1], Fa, QLa, fts, H, c, R, rst, chunks, n, D, d)
    (fm, fL), (sm, sL), nll, fobj, sobj, ssq = _expected(x0, dtm, dom, pl["C0"], pl["P"])
    _check(om, sm, 1e-10, "smoothed means")
    assert _covd(oL, sL) <= 1e-10
    _check(osc[0], nll, 1e-10, "nll")
    _check(osc[1], sobj, 1e-10, "smoother objective")
    _check(osc[3], fobj, 1e-10, "filter objective")
    # sigma^2 whitens with P11^{-T} (the reference's quirk, pof/utils.py:110-112);
    # for d >= 2 that depends on rounding-level sign choices inside tria
    # (LAPACK's dnrm2 and the loops here round differently), so d = 1 only
    if d == 1:
        _check(osc[2], ssq, 1e-10, "sigma^2")
    # filter alone, then smoother alone from the filtered states
    om0, oL0, osc0 = _run(dense_cpu, 0, x0[0], x0[1], Fa, QLa, fts, H, c, R, rst, chunks, n, D, d)
    _check(om0, fm, 1e-10, "filtered means")
    assert _covd(oL0, fL) <= 1e-10
    _check(osc0[1], fobj, 1e-10, "filter objective as obj")
    om2, oL2, osc2 = _run(dense_cpu, 2, om0, oL0, Fa, QLa, fts, None, None, None, 0, chunks, n, D, d)
    _check(om2, sm, 1e-10, "smoothed means (smoother alone)")
    assert _covd(oL2, sL) <= 1e-10
    _check(osc2[1], sobj, 1e-10, "smoother objective (smoother alone)")


def test_dense_chunk_plan(dense_cpu):
    """Chunks never empty: P = ceil(n / C0) after C0 = ceil(n / P_requested);
    the last chunk holds n - (P - 1) C0 >= 1 steps."""
    for n in (1, 2, 7, 64, 100, 4096, 4097):
        for req in (0, 1, 3, 64, 200):
            pl = _plan(dense_cpu, 1, n, 40, 4, req)
            assert 1 <= pl["P"] <= max(1, min(n, req if req else 64))
            assert (pl["P"] - 1) * pl["C0"] < n <= pl["P"] * pl["C0"]
            assert pl["last"] == n - (pl["P"] - 1) * pl["C0"]
            assert 1 <= pl["S"] <= n
