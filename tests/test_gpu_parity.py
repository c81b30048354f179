"""libpof (CUDA, sm_103a) against the NumPy float64 oracle on identical
inputs.  Tolerances: means and covariances (compared as L L^T, square roots
are sign/rotation ambiguous) 1e-10 relative (normwise); NLL and objectives
1e-10 relative; sigma^2 1e-10 relative for d = 1; for d >= 2 sigma^2 is
checked as a formula on the kernel's own filtered states (the reference's
whiten quirk, pof/utils.py:110-112, makes it depend on rounding-level sign
choices, see test_sigma_squared_formula)."""

import numpy as np
import pytest
import torch

from oracle import filtsmooth as ofs, ivp as oivp, solver as osolver
from oracle.scan import sequential_scan
from pof import _lib, ivp as pivp, parallel_filtsmooth as pfs, sequential_filtsmooth as sfs, solver as psolver
from pof.utils import MVNSqrt
from pof.transitions import TransitionModel
from pof.observations import AffineModel

pytestmark = pytest.mark.gpu

TOL = 1e-10


def T(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def N_(x):
    return x.detach().cpu().numpy()


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def covrel(a, b):
    A = a @ np.swapaxes(a, -1, -2)
    B = b @ np.swapaxes(b, -1, -2)
    return rel(A, B)


def close(x, ref, alt):
    """|x - ref| within 1e-10 relative, or within 10x the spread between two
    bracketings of the reference's own arithmetic (its associative-scan tree
    and the sequential filter/smoother): scalars such as the NLL sum terms
    r^2 / S whose innovations r are differences of O(1) quantities, so their
    rounding error is set by the conditioning, not by the implementation."""
    return abs(float(x) - ref) <= max(TOL * abs(ref), 10.0 * abs(ref - alt), 1e-300)


PROBLEMS = {
    "logistic_q2": (lambda: oivp.logistic(r=3.0), 77, 2, 30),
    "lv_q1": (lambda: oivp.lotkavolterra(), 50, 1, 30),
    "vdp_q3": (lambda: oivp.vanderpol(stiffness_constant=1.0), 130, 3, 30),
    "fhn_q3": (lambda: oivp.fhn_classic(tmax=10.0), 200, 3, 40),
    "rigid_q2": (lambda: oivp.rigid_body(), 100, 2, 30),
    "hh_q1": (lambda: oivp.henonheiles(tmax=10.0), 64, 1, 30),
    "logistic_q5": (lambda: oivp.logistic(r=3.0), 300, 5, 30),
}


def problem(key):
    ivpf, N, q, iters = PROBLEMS[key]
    ivp = ivpf()
    ts = np.linspace(ivp.t0, ivp.tmax, N)
    states, info, st = osolver.solve(ivp, ts, q, init="constant", maxiters=iters, return_full=True)
    dom = osolver.linearize_at_previous_states(st, states[0])
    return st, (st.F, st.QL), dom


def gpu_args(st, dtm, dom):
    x0 = MVNSqrt(T(st.x0[0]), T(st.x0[1]))
    gdtm = TransitionModel(T(dtm[0]), T(dtm[1]))
    gdom = AffineModel(T(dom[0]), T(dom[1]), T(dom[2]))
    return x0, gdtm, gdom


@pytest.mark.parametrize("key", list(PROBLEMS))
def test_linear_filtsmooth_parity(key):
    st, dtm, dom = problem(key)
    (om, oL), onll, oobj, ossq = ofs.linear_filtsmooth(st.x0, dtm, dom)
    (_, _), sell, sobj, sssq = ofs.sequential_linear_filtsmooth(st.x0, dtm, dom)
    (gm, gL), gnll, gobj, gssq = pfs.linear_filtsmooth(*gpu_args(st, dtm, dom))
    gm, gL = N_(gm), N_(gL)
    assert rel(gm, om) <= TOL
    assert covrel(gL, oL) <= TOL
    assert close(gnll, onll, -sell)
    assert close(gobj, oobj, sobj)
    if dom[1].shape[-1] == 1:
        assert close(gssq, ossq, sssq)


@pytest.mark.parametrize("key", ["lv_q1", "vdp_q3", "fhn_q3", "rigid_q2", "hh_q1"])
def test_sigma_squared_d_ge_2(key):
    """For d >= 2 the reference's sigma^2 (filter.py:105-114) whitens with
    L^{-T} (utils.py:110-112): each step's term depends on the column signs
    of its observation chol, and for the rank-deficient filtered covariances
    of the noiseless update those signs follow rounding noise.  The kernel's
    value must lie in the range the reference's formula spans over those
    signs (oracle.filtsmooth.sigma_squared_envelope)."""
    st, dtm, dom = problem(key)
    (fm, fL), _, _, _ = ofs.linear_noiseless_filtering(st.x0, dtm, dom)
    lo, hi = ofs.sigma_squared_envelope(dtm, dom, fm, fL)
    (_, _), _, _, gssq = pfs.linear_noiseless_filtering(*gpu_args(st, dtm, dom))
    g = float(gssq)
    assert lo * (1 - 1e-9) <= g <= hi * (1 + 1e-9)


@pytest.mark.parametrize("key", ["logistic_q2", "vdp_q3", "fhn_q3"])
def test_filtering_and_smoothing_entry_points(key):
    st, dtm, dom = problem(key)
    (fm, fL), fnll, fobj, _ = ofs.linear_noiseless_filtering(st.x0, dtm, dom)
    (qm, qL), qell, _ = ofs.linear_noiseless_filter(st.x0, dtm, dom)
    qobj = ofs.filter_objective(dtm, qm)
    x0, gdtm, gdom = gpu_args(st, dtm, dom)
    (gm, gL), gnll, gobj, _ = pfs.linear_noiseless_filtering(x0, gdtm, gdom)
    assert rel(N_(gm), fm) <= TOL and covrel(N_(gL), fL) <= TOL
    assert close(gnll, fnll, -qell)
    assert close(gobj, fobj, qobj)
    # the smoother alone, from the oracle's filtered trajectory
    (sm, sL), sobj = ofs.smoothing(dtm, (fm, fL))
    (hm, hL), hobj = pfs.smoothing(gdtm, MVNSqrt(T(fm), T(fL)))
    assert rel(N_(hm), sm) <= TOL and covrel(N_(hL), sL) <= TOL
    assert abs(float(hobj) - sobj) <= TOL * abs(sobj)


@pytest.mark.parametrize("key", ["logistic_q2", "vdp_q3", "rigid_q2"])
def test_sequential_twin_parity(key):
    st, dtm, dom = problem(key)
    (om, oL), oell, oobj, ossq = ofs.sequential_linear_filtsmooth(st.x0, dtm, dom)
    (_, _), pnll, pobj, pssq = ofs.linear_filtsmooth(st.x0, dtm, dom)
    (gm, gL), gell, gobj, gssq = sfs.linear_filtsmooth(*gpu_args(st, dtm, dom))
    assert rel(N_(gm), om) <= TOL and covrel(N_(gL), oL) <= TOL
    assert close(gell, oell, -pnll)
    assert close(gobj, oobj, pobj)
    if dom[1].shape[-1] == 1:
        assert close(gssq, ossq, pssq)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 9, 31, 32, 33, 35, 257, 5001])
def test_ragged_sizes(n):
    """Chunk and level boundaries: n not a multiple of the chunk sizes, one
    step, several hierarchy levels."""
    ivp = oivp.logistic(r=3.0)
    ts = np.linspace(0.0, 1.0, n + 1)
    st = osolver.set_up_solver(ivp, ts, 2)
    states = osolver.get_initial_trajectory(st, "constant")
    dom = osolver.linearize_at_previous_states(st, states[0])
    dtm = (st.F, st.QL)
    (om, oL), onll, oobj, ossq = ofs.linear_filtsmooth(st.x0, dtm, dom)
    (_, _), sell, sobj, sssq = ofs.sequential_linear_filtsmooth(st.x0, dtm, dom)
    (gm, gL), gnll, gobj, gssq = pfs.linear_filtsmooth(*gpu_args(st, dtm, dom))
    assert rel(N_(gm), om) <= TOL and covrel(N_(gL), oL) <= TOL
    assert close(gnll, onll, -sell)
    assert close(gobj, oobj, sobj)
    assert close(gssq, ossq, sssq)


@pytest.mark.parametrize("key,ks", [("fhn_q3", "4"), ("vdp_q3", "-1"), ("logistic_q5", "3"), ("rigid_q2", "-1")])
def test_parallel_top_matches_tree(key, ks, monkeypatch):
    """The binary tree to the end (the default) and the top level scanned in
    parallel (POF_KS: -1 the lane-count rule, else the largest such level)
    are two bracketings of the same scan: both within the parity tolerance of
    the oracle, and of each other."""
    st, dtm, dom = problem(key)
    (om, oL), onll, oobj, _ = ofs.linear_filtsmooth(st.x0, dtm, dom)
    (_, _), sell, sobj, _ = ofs.sequential_linear_filtsmooth(st.x0, dtm, dom)
    args = gpu_args(st, dtm, dom)
    (am, aL), anll, aobj, _ = pfs.linear_filtsmooth(*args)
    monkeypatch.setenv("POF_KS", ks)
    (bm, bL), bnll, bobj, _ = pfs.linear_filtsmooth(*args)
    for m, L, nll, obj in ((am, aL, anll, aobj), (bm, bL, bnll, bobj)):
        assert rel(N_(m), om) <= TOL and covrel(N_(L), oL) <= TOL
        assert close(nll, onll, -sell)
        assert close(obj, oobj, sobj)
    assert rel(N_(am), N_(bm)) <= TOL and covrel(N_(aL), N_(bL)) <= TOL


@pytest.mark.parametrize("per_step", [False, True])
def test_unstructured_models(per_step):
    """A TransitionModel whose F is dense and Q_L not triangular, and a
    nonzero, non-triangular observation noise: the kernels detect that the
    zero patterns they exploit for the IWP prior (block-upper-triangular F,
    lower-triangular Q_L, R = 0) are absent and run the dense forms (D = 8,
    team kernels; constant and per-step models)."""
    rng = np.random.default_rng(5)
    n, D, d = 300, 8, 2
    F0 = np.eye(D) + 0.05 * rng.standard_normal((D, D))
    Q0 = 0.5 * np.eye(D) + 0.1 * rng.standard_normal((D, D))
    if per_step:
        F = F0 + 0.01 * rng.standard_normal((n, D, D))
        QL = Q0 + 0.01 * rng.standard_normal((n, D, D))
    else:
        F = np.broadcast_to(F0, (n, D, D)).copy()
        QL = np.broadcast_to(Q0, (n, D, D)).copy()
    H = rng.standard_normal((n, d, D))
    c = 0.1 * rng.standard_normal((n, d))
    R = 0.1 * rng.standard_normal((n, d, d))
    x0 = (rng.standard_normal(D), 0.3 * np.eye(D) + 0.05 * np.tril(rng.standard_normal((D, D))))
    (om, oL), onll, oobj, _ = ofs.linear_filtsmooth(x0, (F, QL), (H, c, R))
    (_, _), sell, sobj, _ = ofs.sequential_linear_filtsmooth(x0, (F, QL), (H, c, R))
    gx0 = MVNSqrt(T(x0[0]), T(x0[1]))
    gdtm = TransitionModel(T(F), T(QL)) if per_step else TransitionModel(T(F0), T(Q0))
    (gm, gL), gnll, gobj, _ = pfs.linear_filtsmooth(gx0, gdtm, AffineModel(T(H), T(c), T(R)))
    assert rel(N_(gm), om) <= TOL and covrel(N_(gL), oL) <= TOL
    assert close(gnll, onll, -sell)
    assert close(gobj, oobj, sobj)


def test_deterministic():
    st, dtm, dom = problem("fhn_q3")
    args = gpu_args(st, dtm, dom)
    a = pfs.linear_filtsmooth(*args)
    b = pfs.linear_filtsmooth(*args)
    assert torch.equal(a[0].mean, b[0].mean) and torch.equal(a[0].chol, b[0].chol)
    assert float(a[1]) == float(b[1]) and float(a[2]) == float(b[2]) and float(a[3]) == float(b[3])


SOLVES = [
    ("logistic", lambda: (pivp.logistic(r=3.0), oivp.logistic(r=3.0)), 200, 3),
    ("logistic_ref", lambda: (pivp.logistic(), oivp.logistic()), 64, 2),
    ("vdp0", lambda: (pivp.vanderpol(stiffness_constant=1.0), oivp.vanderpol(stiffness_constant=1.0)), 128, 3),
    ("rigid", lambda: (pivp.rigid_body(), oivp.rigid_body()), 128, 2),
    ("lv", lambda: (pivp.lotkavolterra(), oivp.lotkavolterra()), 256, 1),
    ("logistic_q4", lambda: (pivp.logistic(), oivp.logistic()), 150, 4),
]


@pytest.mark.parametrize("name,mk,N,q", SOLVES)
def test_solve_parity(name, mk, N, q):
    """pof.solver.solve runs the whole IEKS loop in libpof: same iteration
    count as the oracle, means and covariances within 1e-10."""
    p, o = mk()
    ts = np.linspace(o.t0, o.tmax, N)
    (om, oL), oinfo = osolver.solve(o, ts, q, init="constant", maxiters=1000)
    (sm, sL), sinfo = osolver.solve(o, ts, q, init="constant", maxiters=1000, scan=sequential_scan)
    out, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=q, init="constant", maxiters=1000)
    assert int(info["iterations"]) == oinfo["iterations"]
    # the IEKS fixed point amplifies rounding: within 1e-10 or 10x the spread
    # between the reference's tree order and a sequential order
    assert rel(N_(out.mean), om) <= max(TOL, 10 * rel(sm, om))
    # chol_covs carry the calibration factor sigma^2 (solver.py:66-69); compare
    # the covariances per unit sigma^2 (see test_sigma_squared_d_ge_2)
    gs, os_, ss_ = float(info["sigma_squared"]), oinfo["sigma_squared"], sinfo["sigma_squared"]
    assert covrel(N_(out.chol) / gs, oL / os_) <= max(TOL, 10 * covrel(sL / ss_, oL / os_))
    if o.y0.shape[0] == 1:
        assert close(gs, os_, ss_)
    assert close(info["obj"], oinfo["obj"], sinfo["obj"])
    assert close(info["nll"], oinfo["nll"], sinfo["nll"])


def test_solve_user_field_matches_builtin():
    """A plain torch vector field (linearized with torch.func on the GPU)
    gives the built-in field's result: the same iteration count, means within
    1e-10 or 10x the change of the oracle's result when its field is
    perturbed by one unit in the last place (the two linearizations differ
    by rounding, and this IEKS fixed point -- a solution decaying to 1e-7 --
    amplifies a relative 2^-52 in f to ~1.5e-10 in the means)."""
    p, o = pivp.logistic(r=3.0), oivp.logistic(r=3.0)
    ts = np.linspace(0.0, 10.0, 100)

    def f(t, y):
        return 3.0 * y * (1 - y)

    a, ia = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=3, init="constant")
    b, ib = psolver.solve(f=f, y0=p.y0, ts=ts, order=3, init="constant")
    (om, _), _ = osolver.solve(o, ts, 3, init="constant")
    o_ulp = o._replace(components=lambda y: [3.0 * y[0] * (1 - y[0]) * (1 + 2.0**-52)])
    (um, _), _ = osolver.solve(o_ulp, ts, 3, init="constant")
    assert int(ia["iterations"]) == int(ib["iterations"]), (int(ia["iterations"]), int(ib["iterations"]))
    d, tol = rel(N_(b.mean), N_(a.mean)), max(TOL, 10 * rel(um, om))
    assert d <= tol, (d, tol)


@pytest.mark.parametrize("init", ["prior", "coarse"])
def test_solve_other_inits(init):
    p, o = pivp.logistic(), oivp.logistic()
    ts = np.linspace(0.0, 10.0, 60)
    (om, oL), oinfo = osolver.solve(o, ts, 2, init=init, maxiters=1000)
    out, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=2, init=init, maxiters=1000)
    assert int(info["iterations"]) == oinfo["iterations"]
    assert rel(N_(out.mean), om) <= 1e-9


def test_sequential_solves():
    p, o = pivp.vanderpol(stiffness_constant=1.0), oivp.vanderpol(stiffness_constant=1.0)
    ts = np.linspace(0.0, 6.3, 100)
    (om, oL), oinfo = osolver.sequential_eks_solve(o, ts, 3)
    out, info = psolver.sequential_eks_solve(f=p.f, y0=p.y0, ts=ts, order=3)
    assert rel(N_(out.mean), om) <= TOL
    gs, os_ = float(info["sigma_squared"]), oinfo["sigma_squared"]
    assert covrel(N_(out.chol) / gs**0.5, oL / os_**0.5) <= TOL
    (sm, sL), sinfo = osolver.solve(o, ts, 3, init="constant", sequential=True, maxiters=1000)
    out2, info2 = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=3, init="constant", sequential=True, maxiters=1000)
    assert int(info2["iterations"]) == sinfo["iterations"]
    assert rel(N_(out2.mean), sm) <= TOL
