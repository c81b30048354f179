"""The NumPy float64 oracle against the reference's own tests and published
float64 results (CPU only)."""

import json
import os

import numpy as np
import pytest

from oracle import blocked, core, filtsmooth as ofs, ivp as oivp, scan, solver as osolver, taylor

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "v100_ieks.json")))

CTORS = {
    "logistic": lambda: oivp.logistic(),
    "vdp0": lambda: oivp.vanderpol(stiffness_constant=1.0),
    "rigidbody": lambda: oivp.rigid_body(),
    "henonheiles": lambda: oivp.henonheiles(tmax=10.0),
    "fhn": lambda: oivp.fitzhughnagumo(),
}


def _reference_solution(name, ivp, ts):
    if name == "logistic":
        return (1.0 / (1.0 + (1.0 / 0.01 - 1.0) * np.exp(-ts)))[:, None]
    from scipy.integrate import solve_ivp

    sol = solve_ivp(lambda t, y: ivp.f(t, y), ivp.t_span, ivp.y0, method="DOP853", rtol=1e-13, atol=1e-16,
                    dense_output=True)
    return sol.sol(ts).T


def _rows(setup, nmax):
    return [r for r in GOLD["rows"] if r["setup"] == setup and r["N"] <= nmax]


CASES = [(r["setup"], r["N"], r["q"]) for s, nmax in (("logistic", 256), ("vdp0", 256), ("rigidbody", 256),
                                                    ("henonheiles", 128)) for r in _rows(s, nmax)]


@pytest.mark.parametrize("setup,N,q", CASES)
def test_oracle_matches_published_v100_float64(setup, N, q):
    """Iteration count and trajectory RMSE of solve(init='constant',
    maxiters=1000) equal the reference's published float64 results
    (experiments/3_work_precision_diagram/data/*_V100*.csv)."""
    row = next(r for r in GOLD["rows"] if (r["setup"], r["N"], r["q"]) == (setup, N, q))
    ivp = CTORS[setup]()
    ts = np.linspace(ivp.t0, ivp.tmax, N)
    ys, info = osolver.solve(ivp, ts, q, init="constant", maxiters=1000)
    assert info["iterations"] == row["iterations"]
    yref = _reference_solution(setup, ivp, ts)
    rmse = np.mean(np.linalg.norm(ys[0] - yref, axis=1))
    # the reference's own error reference (Kvaerno5, rtol 1e-13) floors near 1e-11
    if row["rmse_traj"] > 1e-9:
        assert abs(rmse - row["rmse_traj"]) <= 1e-3 * row["rmse_traj"] + 3e-11
    else:
        assert rmse < 1e-9


def _trivial_model():
    """tests/test_filtsmooth.py:16-33: q = 0, d = 1, obs = E0 x, x0 = 0."""
    d, q = 1, 0
    E0 = core.projection_matrix(d, q, 0)
    ts = np.arange(10.0)
    F, QL = core.discretize_transitions(d, q, ts[1:] - ts[:-1])
    x0 = (np.zeros(1), np.zeros((1, 1)))
    n = F.shape[0]
    H = np.repeat(E0[None], n, 0)
    c = np.zeros((n, 1))
    R = np.zeros((n, 1, 1))
    return x0, (F, QL), (H, c, R)


def test_sequential_equals_parallel_trivial_model():
    """The reference's cross-implementation identity (tests/test_filtsmooth.py:41-62)."""
    x0, dtm, dom = _trivial_model()
    (fm, fL), _, _ = ofs.linear_noiseless_filter(x0, dtm, dom)
    (sm, sL), _ = ofs.sequential_smoothing(dtm, (fm, fL))
    (pm, pL), _, _, _ = ofs.linear_noiseless_filtering(x0, dtm, dom)
    (psm, psL), _ = ofs.smoothing(dtm, (pm, pL))
    assert np.array_equal(fm, pm) and np.array_equal(fL, pL)
    assert np.array_equal(sm, psm) and np.array_equal(sL, psL)


@pytest.mark.parametrize("dim", [1, 3, 5])
@pytest.mark.parametrize("order", [1, 3, 5])
def test_projection_matrix(dim, order):
    """tests/test_transtions.py:19-32."""
    D = dim * (order + 1)
    E0 = core.projection_matrix(dim, order, 0)
    E1 = core.projection_matrix(dim, order, 1)
    assert E0.shape == (dim, D) and E1.shape == (dim, D)
    x = np.random.default_rng(0).uniform(size=D)
    assert np.array_equal(E0 @ x, x[0:: order + 1])
    assert np.array_equal(E1 @ x, x[1:: order + 1])


def test_discretize_shapes():
    """tests/test_transtions.py:35-44."""
    F, QL = core.non_preconditioned_discretize(2, 3, 0.1)
    assert F.shape == (8, 8) and QL.shape == (8, 8)


@pytest.mark.parametrize("ivpf,q", [(oivp.logistic, 3), (oivp.fhn_classic, 4), (oivp.lotkavolterra, 2),
                                    (oivp.threebody, 3), (oivp.henonheiles, 5)])
def test_taylor_init_residual(ivpf, q):
    """x0 from Taylor mode satisfies E1 x0 = f(E0 x0) and the chain rule
    for the second derivative (J f)."""
    ivp = ivpf()
    derivs = taylor.taylor_derivatives(ivp.components, ivp.y0, q)
    y, dy, ddy = derivs[0], derivs[1], derivs[2]
    assert np.allclose(dy, ivp.f(None, y), rtol=1e-14, atol=1e-14)
    assert np.allclose(ddy, ivp.jac(y) @ ivp.f(None, y), rtol=1e-12, atol=1e-12)


def test_linearize_identity():
    """tests/test_observations.py:23-33: H m + b == f(m), cholR == 0."""
    ivp = oivp.fhn_classic()
    st = osolver.set_up_solver(ivp, np.linspace(0, 10, 11), 3)
    m = np.random.default_rng(1).normal(size=(5, 8))
    H, c, R = osolver.linearize(st, m)
    assert H.shape == (5, 2, 8) and c.shape == (5, 2) and R.shape == (5, 2, 2)
    assert np.all(R == 0)
    res = osolver.observation_residual(st, m)
    assert np.allclose(np.einsum("nij,nj->ni", H, m) + c, res, rtol=1e-13, atol=1e-13)


def _converged_problem(ivp, N, q, iters):
    ts = np.linspace(ivp.t0, ivp.tmax, N)
    states, info, st = osolver.solve(ivp, ts, q, init="constant", maxiters=iters, return_full=True)
    dom = osolver.linearize_at_previous_states(st, states[0])
    return st, (st.F, st.QL), dom


def _covd(a, b):
    A = a @ np.swapaxes(a, -1, -2)
    B = b @ np.swapaxes(b, -1, -2)
    return np.abs(A - B).max() / np.abs(B).max()


@pytest.mark.parametrize("ivpf,N,q", [(lambda: oivp.logistic(r=3.0), 77, 2), (oivp.lotkavolterra, 50, 1),
                                      (lambda: oivp.vanderpol(stiffness_constant=1.0), 130, 3)])
@pytest.mark.parametrize("C0,Cs", [(5, (3, 2)), (16, (4,)), (1, (2,) * 12)])
def test_blocked_schedule_equals_reference_scan(ivpf, N, q, C0, Cs):
    """The chunked schedule the kernels run gives the reference scan's
    filtered/smoothed marginals, NLL and objectives to rounding."""
    st, dtm, dom = _converged_problem(ivpf(), N, q, 50)
    (fm, fL), nll, obj, ssq = ofs.linear_noiseless_filtering(st.x0, dtm, dom)
    (bm, bL), bnll, bobj, bssq, _ = blocked.filter_blocked(st.x0, dtm, dom, C0=C0, Cs=Cs)
    assert np.abs(fm - bm).max() <= 1e-12 * np.abs(fm).max()
    assert _covd(bL, fL) <= 1e-12
    assert abs(nll - bnll) <= 1e-11 * abs(nll)
    assert abs(obj - bobj) <= 1e-11 * abs(obj)
    if dom[1].shape[-1] == 1:  # sigma^2 is sign-pattern dependent for d >= 2 (whiten quirk)
        assert abs(ssq - bssq) <= 1e-11 * abs(ssq)
    (sm, sL), sobj = ofs.smoothing(dtm, (fm, fL))
    (bsm, bsL), bsobj = blocked.smoother_blocked(dtm, (bm, bL), C0=C0, Cs=Cs)
    assert np.abs(sm - bsm).max() <= 1e-12 * np.abs(sm).max()
    assert _covd(bsL, sL) <= 1e-12
    assert abs(sobj - bsobj) <= 1e-11 * abs(sobj)


@pytest.mark.parametrize("ivpf,N,q", [(lambda: oivp.logistic(r=3.0), 77, 2),
                                      (lambda: oivp.vanderpol(stiffness_constant=1.0), 130, 3)])
@pytest.mark.parametrize("C0,Cg", [(4, 2), (3, 5), (1, 2), (200, 2)])
def test_segmented_schedule_equals_reference_scan(ivpf, N, q, C0, Cg):
    """The batched solve's schedule (every chunk a conditional fold, groups
    until one element per problem, x0 / terminal injected at the top) gives
    the reference scan's marginals, NLL and objectives to rounding."""
    st, dtm, dom = _converged_problem(ivpf(), N, q, 50)
    (fm, fL), nll, obj, ssq = ofs.linear_noiseless_filtering(st.x0, dtm, dom)
    (bm, bL), bnll, bobj, bssq, _ = blocked.filter_blocked(st.x0, dtm, dom, C0=C0, Cs=(Cg,), segmented=True)
    assert np.abs(fm - bm).max() <= 1e-12 * np.abs(fm).max()
    assert _covd(bL, fL) <= 1e-12
    assert abs(nll - bnll) <= 1e-11 * abs(nll)
    assert abs(obj - bobj) <= 1e-11 * abs(obj)
    if dom[1].shape[-1] == 1:
        assert abs(ssq - bssq) <= 1e-11 * abs(ssq)
    (sm, sL), sobj = ofs.smoothing(dtm, (fm, fL))
    (bsm, bsL), bsobj = blocked.smoother_blocked(dtm, (bm, bL), C0=C0, Cs=(Cg,), segmented=True)
    assert np.abs(sm - bsm).max() <= 1e-12 * np.abs(sm).max()
    assert _covd(bsL, sL) <= 1e-12
    assert abs(sobj - bsobj) <= 1e-11 * abs(sobj)


@pytest.mark.parametrize("ivpf,N,q", [(lambda: oivp.logistic(r=3.0), 77, 2),
                                      (lambda: oivp.vanderpol(stiffness_constant=1.0), 130, 3)])
@pytest.mark.parametrize("C0,Cs,ks_max", [(1, (2,) * 12, 1024), (2, (2,) * 12, 16), (4, (2,) * 12, 3),
                                          (1, (2,) * 12, 37)])
def test_parallel_top_scan_equals_reference_scan(ivpf, N, q, C0, Cs, ks_max):
    """The plain path's schedule with its top level scanned in parallel
    (Kogge-Stone prefix scan of the filter, suffix scan of the smoother after
    pushing the terminal state through the last element) gives the reference
    scan's marginals, NLL and objectives to rounding."""
    st, dtm, dom = _converged_problem(ivpf(), N, q, 50)
    (fm, fL), nll, obj, ssq = ofs.linear_noiseless_filtering(st.x0, dtm, dom)
    (bm, bL), bnll, bobj, bssq, _ = blocked.filter_blocked(st.x0, dtm, dom, C0=C0, Cs=Cs, ks_max=ks_max)
    assert np.abs(fm - bm).max() <= 1e-12 * np.abs(fm).max()
    assert _covd(bL, fL) <= 1e-12
    assert abs(nll - bnll) <= 1e-11 * abs(nll)
    assert abs(obj - bobj) <= 1e-11 * abs(obj)
    (sm, sL), sobj = ofs.smoothing(dtm, (fm, fL))
    (bsm, bsL), bsobj = blocked.smoother_blocked(dtm, (bm, bL), C0=C0, Cs=Cs, ks_max=ks_max)
    assert np.abs(sm - bsm).max() <= 1e-12 * np.abs(sm).max()
    assert _covd(bsL, sL) <= 1e-12
    assert abs(sobj - bsobj) <= 1e-11 * abs(sobj)


def test_scan_orders_agree():
    """JAX's odd/even recursion and a left fold give the same prefix sums."""
    rng = np.random.default_rng(0)
    x = rng.normal(size=(37, 3))
    add = lambda a, b: (a[0] + b[0],)  # noqa: E731
    (a,) = scan.associative_scan(add, (x,))
    (b,) = scan.sequential_scan(add, (x,))
    assert np.allclose(a, np.cumsum(x, 0)) and np.allclose(b, np.cumsum(x, 0))
    (r,) = scan.associative_scan(add, (x,), reverse=True)
    assert np.allclose(r, np.cumsum(x[::-1], 0)[::-1])


@pytest.mark.parametrize("ivpf,N,q", [(lambda: oivp.fhn_classic(tmax=10.0), 200, 3), (oivp.lotkavolterra, 50, 1),
                                      (oivp.rigid_body, 100, 2)])
def test_sigma_squared_envelope_contains_reference_orders(ivpf, N, q):
    """sigma^2 of d >= 2 problems differs between evaluation orders of the
    reference's own arithmetic (whiten quirk); all of them lie in the sign
    envelope that the GPU tests check against."""
    from oracle.scan import sequential_scan

    st, dtm, dom = _converged_problem(ivpf(), N, q, 30)
    (fm, fL), _, _, t = ofs.linear_noiseless_filtering(st.x0, dtm, dom)
    _, _, _, s = ofs.linear_noiseless_filtering(st.x0, dtm, dom, scan=sequential_scan)
    _, _, _, b, _ = blocked.filter_blocked(st.x0, dtm, dom, C0=4, Cs=(8,) * 24)
    lo, hi = ofs.sigma_squared_envelope(dtm, dom, fm, fL)
    for v in (t, s, b):
        assert lo * (1 - 1e-9) <= v <= hi * (1 + 1e-9)


def test_quadratic_penalty_iterator_escapes_a_spurious_fixed_point():
    """What the quadratic-penalty IEKS is for (iterators.py:44-106): on the
    logistic ODE y' = 3 y (1 - y), y(0) = 0.01, on 60 grid points over
    [0, 10], q = 2, the plain IEKS from the constant start stops after four
    iterations at the fixed point y = 0, while the penalty continuation
    (reg 1e20 -> 0 over 40 stages) ends on the solution."""
    from oracle import ivp as oivp, solver as osolver

    o = oivp.logistic(r=3.0)
    ts = np.linspace(0.0, 10.0, 60)
    exact = 1.0 / (1.0 + (1.0 / 0.01 - 1.0) * np.exp(-3.0 * ts))
    (om, _), info = osolver.solve(o, ts, 2, init="constant")
    assert info["iterations"] == 4 and abs(om[-1, 0]) < 1e-6
    it, st = osolver.qpm_ieks_iterator(o, ts, 2, init="constant")
    regs = []
    for s, _, _, reg in it:
        regs.append(reg)
        last = s
    ys = last[0] @ st.E0.T
    assert regs[0] == 1e20 and regs[-1] == 0.0 and len(regs) >= 42
    assert np.abs(ys[:, 0] - exact).max() < 1e-4


@pytest.mark.parametrize("D,d,n", [(8, 2, 61), (6, 3, 40), (4, 1, 33)])
@pytest.mark.parametrize("C0,Cs,segmented,ks_max", [(4, (2,) * 8, False, 0), (3, (3, 2), False, 0),
                                                     (5, (2,), True, 0), (1, (2,) * 8, False, 16)])
def test_blocked_schedules_on_unstructured_per_step_models(D, d, n, C0, Cs, segmented, ks_max):
    """The kernels' schedules (chunked tree, batched segmentation, parallel
    top) restated in oracle/blocked.py, on models with none of the IWP
    prior's zero patterns: a dense F and a full lower Q_L per step, a nonzero
    observation noise per step, x0 with a full chol.  Same filtered and
    smoothed marginals, NLL and objectives as the reference scan."""
    rng = np.random.default_rng(1000 * D + n)
    F = rng.standard_normal((n, D, D)) / np.sqrt(D) + 0.5 * np.eye(D)
    QL = np.tril(rng.standard_normal((n, D, D))) * 0.2 + 0.5 * np.eye(D)
    H = rng.standard_normal((n, d, D))
    c = rng.standard_normal((n, d))
    R = np.tril(rng.standard_normal((n, d, d))) * 0.1 + 0.3 * np.eye(d)
    x0 = (rng.standard_normal(D), np.tril(rng.standard_normal((D, D))) * 0.3 + np.eye(D))
    dtm, dom = (F, QL), (H, c, R)
    (fm, fL), nll, obj, _ = ofs.linear_noiseless_filtering(x0, dtm, dom)
    (bm, bL), bnll, bobj, _, _ = blocked.filter_blocked(x0, dtm, dom, C0=C0, Cs=Cs, segmented=segmented,
                                                         ks_max=ks_max)
    assert np.abs(fm - bm).max() <= 1e-10 * np.abs(fm).max()
    assert _covd(bL, fL) <= 1e-10
    assert abs(nll - bnll) <= 1e-10 * abs(nll) and abs(obj - bobj) <= 1e-10 * abs(obj)
    (sm, sL), sobj = ofs.smoothing(dtm, (fm, fL))
    (bsm, bsL), bsobj = blocked.smoother_blocked(dtm, (bm, bL), C0=C0, Cs=Cs, segmented=segmented, ks_max=ks_max)
    assert np.abs(sm - bsm).max() <= 1e-10 * np.abs(sm).max()
    assert _covd(bsL, sL) <= 1e-10
    assert abs(sobj - bsobj) <= 1e-10 * abs(sobj)
