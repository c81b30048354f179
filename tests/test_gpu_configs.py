"""libpof on the benchmark configurations themselves, against the float64
oracle (fixture ``tests/golden/config_goldens.npz``, made by
``tests/golden/make_config_goldens.py``, for the solves that take the oracle
minutes; the oracle itself for the rest).

Tolerance rule of every comparison here: the GPU result is within 1e-10
relative (normwise max) of the oracle's reference-order result, or within
10x the spread between two reference-faithful orders of the oracle (its
associative-scan tree and the sequential filter/smoother) when that spread
is larger -- an IEKS fixed point, or one ill-conditioned filter/smoother
pass, amplifies rounding by the conditioning of the problem, and no
bracketing can agree with the reference better than the reference's own two
orders agree.  Each test prints the tolerance it used, and fails when it
exceeds 1e-8 unless the case is named in ILL_CONDITIONED with the measured
spread that puts it there.

Iteration counts: the reference's criterion (pof/convergence_criteria.py:4-13)
stops on a relative objective change below 1e-6; where the two oracle orders
stop at the same iteration on a well-conditioned case, the GPU must too;
where they do not (the count itself is decided by rounding: logistic q = 5,
N = 2^10 stops after 38 iterations in one order and 74 in the other), the
test prints the counts and checks the solution only.
"""

import os

import numpy as np
import pytest
import torch

from oracle import filtsmooth as ofs, ivp as oivp, solver as osolver
from pof import _lib, ivp as pivp, parallel_filtsmooth as pfs, solver as psolver, step as pstep
from pof.convenience import set_up_solver
from pof.observations import AffineModel
from pof.transitions import TransitionModel
from pof.utils import MVNSqrt

pytestmark = pytest.mark.gpu

TOL = 1e-10
CAP = 1e-8
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config_goldens.npz")

# Cases whose two oracle orders disagree by more than CAP / 10 from the same
# input, with the spread measured by the oracle (tree vs sequential order).
# FitzHugh-Nagumo over t in [0, 100]: one IEKS iteration from the oracle's
# iterates 20 and 400 of its solve is ill-conditioned (at its converged
# iterate 656 the orders agree to 4e-14 and the 1e-10 bound holds).  The
# logistic sweep: two grids whose IEKS fixed point amplifies rounding.
ILL_CONDITIONED = {
    "fhn_n1000_step_20": "oracle orders differ by 2.6e-6 after one iteration",
    "fhn_n1000_step_400": "oracle orders differ by 4.1e-4 after one iteration",
    "log_q2_N4096": "oracle orders' solutions differ by 2.8e-9",
    "log_q3_N4096": "oracle orders' solutions differ by 5.0e-8",
}


def T(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def N_(x):
    return x.detach().cpu().numpy()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def covrel(a, b):
    A = a @ np.swapaxes(a, -1, -2)
    B = b @ np.swapaxes(b, -1, -2)
    return rel(A, B)


def eff_tol(name, spread):
    tol = max(TOL, 10.0 * spread)
    print("[%s] effective tolerance %.3g (oracle order spread %.3g)" % (name, tol, spread))
    if tol > CAP:
        assert name in ILL_CONDITIONED, "%s: tolerance %.3g above %.0e and not listed as ill-conditioned" % (
            name, tol, CAP)
    return tol


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def obj_margin(trace, k):
    """Relative objective change at iteration k (1-based) of a trace of
    (obj, nll, ssq) rows: the quantity crit compares with 1e-6."""
    if k < 2:
        return float("inf")
    o, oo = trace[k - 1][0], trace[k - 2][0]
    return abs(o - oo) / abs(o)


# ---------------------------------------------------------------------------
# FitzHugh-Nagumo, a = b = 0.2, c = 3, y0 = (-1, 1), t in [0, 100], N = 1000,
# q = 3 (D = 8), constant init: the reference's CPU configuration
# ---------------------------------------------------------------------------

def _fhn_setup():
    o = oivp.fhn_classic()
    ts = np.linspace(0.0, 100.0, 1000)
    return o, ts, osolver.set_up_solver(o, ts, 3)


def _gpu_step(ts, m_in):
    """pof.step.ieks_step on the GPU from the preconditioned means m_in."""
    p = pivp.fhn_classic()
    setup = set_up_solver(f=p.f, y0=p.y0, ts=ts, order=3)
    D = m_in.shape[-1]
    return pstep.ieks_step(om=setup["om"], dtm=setup["dtm"], x0=setup["x0"],
                           states=MVNSqrt(T(m_in), T(np.zeros(m_in.shape + (D,)))))


def _check_step(name, st, ts, m_in):
    states_in = (m_in, np.zeros(m_in.shape + (m_in.shape[-1],)))
    (om, oL), onll, oobj, ossq = osolver.ieks_step(st, states_in)
    (sm, sL), snll, sobj, sssq = osolver.ieks_step(st, states_in, sequential=True)
    gs, gnll, gobj, gssq = _gpu_step(ts, m_in)
    spread = rel(sm, om)
    tol = eff_tol(name, spread)
    print("[%s] gpu vs oracle tree %.3g" % (name, rel(N_(gs.mean), om)))
    assert rel(N_(gs.mean), om) <= tol, (rel(N_(gs.mean), om), tol)
    # covariances per unit sigma^2 (sigma^2 of d >= 2 depends on rounding-level signs)
    ctol = max(tol, 10 * covrel(sL / sssq**0.5, oL / ossq**0.5))
    assert covrel(N_(gs.chol) / float(gssq) ** 0.5, oL / ossq**0.5) <= ctol
    assert abs(float(gobj) - oobj) <= max(tol, 10 * abs(sobj - oobj) / abs(oobj)) * abs(oobj)
    return spread


def test_fhn_n1000_first_iteration_matches_oracle():
    """The first IEKS iteration of the configuration (from the constant
    initial trajectory, pof/convenience.py:76-92): the EK1 linearization and
    the filter/smoother pass in libpof equal the oracle within 1e-10, and
    the oracle's two orders agree to 1e-12 there."""
    o, ts, st = _fhn_setup()
    m0 = osolver.get_initial_trajectory(st, "constant")[0]
    assert _check_step("fhn_n1000_step_0", st, ts, m0) <= 1e-12


@pytest.mark.parametrize("k", [20, 400, 656])
def test_fhn_n1000_step_from_oracle_iterates(gold, k):
    """One IEKS iteration from the oracle's own iterate k of this solve (the
    reference's associative-scan order): the GPU's next iterate is within
    10x the spread of the oracle's two orders from the same input."""
    o, ts, st = _fhn_setup()
    _check_step("fhn_n1000_step_%d" % k, st, ts, gold["fhn_m%d" % k])


def test_fhn_n1000_solve(gold):
    """The whole solve (pof.solver.solve, the IEKS loop in libpof).  On this
    configuration the IEKS iteration is ill-conditioned after the first one
    (test_fhn_n1000_step_from_oracle_iterates): from the same iterate, the
    reference's associative-scan and sequential orders give next iterates
    that differ by up to O(1), so the iteration count and the fixed point
    reached are decided by rounding, differently in each order.  Checked:
    the loop stops on the reference's criterion (status converged, finite
    results), and the oracle's two orders agree at iteration 1 and part at
    iteration 2; the counts, objectives and distances are printed."""
    o, ts, st = _fhn_setup()
    p = pivp.fhn_classic()
    out, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=3, init="constant")
    it = int(info["iterations"])
    it_tree, it_seq = (int(x) for x in gold["fhn_iterations"])  # it_seq -1: not in the fixture
    y = N_(out.mean)
    print("[fhn_n1000] iterations: gpu %d, oracle tree %d, oracle sequential %s" % (
        it, it_tree, it_seq if it_seq >= 0 else "n/a"))
    print("[fhn_n1000] final objective: gpu %.6g, oracle tree %.6g (its last change %.3g; crit 1e-6)" % (
        float(info["obj"]), gold["fhn_trace_tree"][it_tree - 1][0], obj_margin(gold["fhn_trace_tree"], it_tree)))
    print("[fhn_n1000] final y vs oracle tree: gpu %.3g" % rel(y, gold["fhn_y_tree"]))
    if "fhn_y_seq" in gold:
        print("[fhn_n1000] oracle sequential vs tree %.3g" % rel(gold["fhn_y_seq"], gold["fhn_y_tree"]))
    assert _lib.solve_status(int(info["status"])) == "converged"
    assert np.isfinite(y).all() and np.isfinite(N_(out.chol)).all()
    assert 1 <= it <= 10_001
    if it_tree == it_seq:
        assert it == it_tree
    # the reference's own two orders agree after the first iteration and
    # part after the second (the reason the count is rounding-decided here)
    states = osolver.get_initial_trajectory(st, "constant")
    a1, _, oa1, _ = osolver.ieks_step(st, states)
    b1, _, ob1, _ = osolver.ieks_step(st, states, sequential=True)
    _, _, oa2, _ = osolver.ieks_step(st, a1)
    _, _, ob2, _ = osolver.ieks_step(st, b1, sequential=True)
    print("[fhn_n1000] oracle objectives, tree / sequential: iteration 1 %.9g / %.9g, iteration 2 %.6g / %.6g" % (
        oa1, ob1, oa2, ob2))
    assert abs(oa1 - ob1) <= 1e-12 * abs(oa1)
    assert abs(oa2 - ob2) > 1e-3 * abs(oa2)


def test_fhn_bench_shape_filtsmooth_matches_oracle():
    """One linear_filtsmooth pass at the benchmark's shape (FitzHugh-Nagumo,
    q = 3, N = 2^16), linearized at the constant initial trajectory: means,
    covariances (L L^T), NLL and objective within 1e-10 of the oracle."""
    o = oivp.fhn_classic()
    N = 2**16
    ts = np.linspace(0.0, 100.0, N)
    st = osolver.set_up_solver(o, ts, 3)
    m0 = osolver.get_initial_trajectory(st, "constant")[0]
    dom = osolver.linearize_at_previous_states(st, m0)
    dtm = (st.F, st.QL)
    (om, oL), onll, oobj, ossq = ofs.linear_filtsmooth(st.x0, dtm, dom)
    x0 = MVNSqrt(T(st.x0[0]), T(st.x0[1]))
    gdtm = TransitionModel(T(st.F[0]), T(st.QL[0]))
    (gm, gL), gnll, gobj, gssq = pfs.linear_filtsmooth(x0, gdtm, AffineModel(*(T(x) for x in dom)))
    print("[fhn_N65536] means %.3g, L L^T %.3g, nll %.3g, obj %.3g" % (
        rel(N_(gm), om), covrel(N_(gL), oL), abs(float(gnll) - onll) / abs(onll),
        abs(float(gobj) - oobj) / abs(oobj)))
    assert rel(N_(gm), om) <= TOL
    assert covrel(N_(gL), oL) <= TOL
    assert abs(float(gnll) - onll) <= TOL * abs(onll)
    assert abs(float(gobj) - oobj) <= TOL * abs(oobj)


# ---------------------------------------------------------------------------
# Logistic y' = 3 y (1 - y), y0 = 0.01, t in [0, 10], q in {1, 2, 3, 5},
# N in {2^10, 2^12, 2^14}: the scan-length sweep
# ---------------------------------------------------------------------------

LOGISTIC = [(q, N) for q in (1, 2, 3, 5) for N in (2**10, 2**12, 2**14)]


@pytest.mark.parametrize("q,N", LOGISTIC)
def test_logistic_sweep_solve(gold, q, N):
    key = "log_q%d_N%d" % (q, N)
    p = pivp.logistic(r=3.0)
    ts = np.linspace(0.0, 10.0, N)
    out, info = psolver.solve(f=p.f, y0=p.y0, ts=ts, order=q, init="constant")
    it = int(info["iterations"])
    it_tree, it_seq = (int(x) for x in gold[key + "_iterations"])
    print("[%s] iterations: gpu %d, oracle tree %d, oracle sequential %d" % (key, it, it_tree, it_seq))
    assert _lib.solve_status(int(info["status"])) == "converged"
    spread = float(gold[key + "_spread"])
    y = N_(out.mean)[gold[key + "_idx"], 0]
    print("[%s] gpu vs oracle tree %.3g" % (key, rel(y, gold[key + "_y"])))
    # the solution: within 1e-10, or 10x the oracle orders' spread
    tol = eff_tol(key, spread)
    assert rel(y, gold[key + "_y"]) <= tol, (rel(y, gold[key + "_y"]), tol)
    ot, os_ = gold[key + "_scalars"][0][0], gold[key + "_scalars"][1][0]
    # the iteration count: the reference's criterion compares a relative
    # objective change with 1e-6 near the fixed point, so where the oracle's
    # two orders stop at different iterations, or the case is listed as
    # ill-conditioned, the count is decided by rounding and only reported
    if it_tree == it_seq and key not in ILL_CONDITIONED:
        assert it == it_tree
        assert abs(float(info["obj"]) - ot) <= max(tol, 10 * abs(os_ - ot) / abs(ot)) * abs(ot)
    else:
        print("[%s] rounding-decided iteration count" % key)
