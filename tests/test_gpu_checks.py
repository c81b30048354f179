"""The bounds-checked build of libpof (-DPOF_CHECKS, built by
pof._build.build(checks=True) as libpof_checked.so): every global index the
kernels derive from sizes and plan tables -- SoA element indices, step
indices of the level-0 chunks, problem indices of the batched plans -- is
tested before its access, and the first failing check's source line is
recorded (pof_checks_read).  Memory sanitizers are not run on these GPUs;
this build stands in for them.  The same kinds of calls as the other GPU
tests -- thread-per-chunk and team kernels, ragged sizes, per-step models,
the Levenberg-Marquardt shape, the IEKS loop as a graph, the sequential
plan, batches and the serving engine -- must record no failure, and give the
normal build's results bit for bit."""

import ctypes

import numpy as np
import pytest
import torch

from oracle import ivp as oivp, solver as osolver
from pof import _build, _lib, batch as pbatch, ivp as pivp, parallel_filtsmooth as pfs, serve, solver as psolver
from pof.observations import AffineModel
from pof.transitions import TransitionModel
from pof.utils import MVNSqrt

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked():
    lib = _lib.load(_build.build(checks=True, verbose=False))
    assert lib.pof_checks_compiled() == 1
    assert _lib.lib().pof_checks_compiled() == 0
    line = ctypes.c_uint64(7)
    assert lib.pof_checks_read(ctypes.byref(line), 1) == 0
    return lib


def _no_failures(lib):
    line = ctypes.c_uint64(0)
    assert lib.pof_checks_read(ctypes.byref(line), 1) == 0
    assert line.value == 0, "bounds check failed at csrc line %d" % line.value


def _both(checked, monkeypatch, fn):
    """fn() with the normal build, then with the checked build."""
    a = fn()
    torch.cuda.synchronize()
    monkeypatch.setattr(_lib, "_lib", checked)
    b = fn()
    torch.cuda.synchronize()
    monkeypatch.undo()
    _no_failures(checked)
    return a, b


def T(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def _filtsmooth_case(ivp, N, q, per_step=False):
    ts = np.linspace(ivp.t0, ivp.tmax, N)
    st = osolver.set_up_solver(ivp, ts, q)
    states = osolver.get_initial_trajectory(st, "constant")
    H, c, R = osolver.linearize_at_previous_states(st, states[0])
    F, QL = (st.F, st.QL) if per_step else (st.F[0], st.QL[0])
    return (MVNSqrt(T(st.x0[0]), T(st.x0[1])), TransitionModel(T(F), T(QL)), AffineModel(T(H), T(c), T(R)))


@pytest.mark.parametrize("name,mk,N,q,per_step", [
    ("logistic_q2_one_step", lambda: oivp.logistic(r=3.0), 2, 2, False),
    ("logistic_q2_ragged", lambda: oivp.logistic(r=3.0), 258, 2, False),
    ("fhn_q3", lambda: oivp.fhn_classic(tmax=10.0), 200, 3, False),
    ("fhn_q3_per_step", lambda: oivp.fhn_classic(tmax=10.0), 131, 3, True),
    ("rigid_q3_D12", lambda: oivp.rigid_body(), 77, 3, False),
])
def test_filtsmooth_checked(checked, monkeypatch, name, mk, N, q, per_step):
    args = _filtsmooth_case(mk(), N, q, per_step)
    a, b = _both(checked, monkeypatch, lambda: pfs.linear_filtsmooth(*args))
    assert torch.equal(a[0].mean, b[0].mean) and torch.equal(a[0].chol, b[0].chol)
    assert float(a[1]) == float(b[1]) and float(a[2]) == float(b[2])


def test_levenberg_marquardt_shape_checked(checked, monkeypatch):
    """(D, d) = (3, 4): more observation rows than states, nonzero noise."""
    rng = np.random.default_rng(1)
    n, D, d = 40, 3, 4
    x0 = MVNSqrt(T(rng.standard_normal(D)), T(0.1 * np.eye(D)))
    dtm = TransitionModel(T(np.eye(D) + 0.1 * np.triu(rng.standard_normal((D, D)))), T(0.3 * np.eye(D)))
    R = np.zeros((n, d, d))
    R[:, 1:, 1:] = np.eye(3)
    dom = AffineModel(T(rng.standard_normal((n, d, D))), T(rng.standard_normal((n, d))), T(R))
    a, b = _both(checked, monkeypatch, lambda: pfs.linear_filtsmooth(x0, dtm, dom))
    assert torch.equal(a[0].mean, b[0].mean) and torch.equal(a[0].chol, b[0].chol)


@pytest.mark.parametrize("sequential", [False, True])
def test_solves_checked(checked, monkeypatch, sequential):
    p = pivp.vanderpol(stiffness_constant=1.0)
    ts = np.linspace(0.0, 6.3, 150)
    a, b = _both(checked, monkeypatch,
                 lambda: psolver.solve(f=p.f, y0=p.y0, ts=ts, order=3, init="constant", sequential=sequential))
    assert torch.equal(a[0].mean, b[0].mean) and int(a[1]["iterations"]) == int(b[1]["iterations"])


def test_batch_and_server_checked(checked, monkeypatch):
    probs = [("vanderpol", (1.0,), [2.0, 0.0], np.linspace(0.0, 6.3, 128)),
             ("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], np.linspace(0.0, 7.0, 301)),
             ("vanderpol", (1.2,), [1.9, 0.1], np.linspace(0.0, 5.0, 17))]
    a, b = _both(checked, monkeypatch, lambda: pbatch.solve_batch(probs, order=3, maxiters=200))
    assert torch.equal(a.mean, b.mean) and torch.equal(a.info["iterations"], b.info["iterations"])

    def served():
        srv = serve.Server(max_requests=4, max_points=1 << 12)
        rids = [srv.submit(nm, p, y0, ts, 3, maxiters=200) for (nm, p, y0, ts) in probs]
        while srv.busy():
            srv.tick()
        out = [srv.result(r)[0][0].clone() for r in rids]
        srv.close()
        return out

    sa, sb = _both(checked, monkeypatch, served)
    assert all(torch.equal(x, y) for x, y in zip(sa, sb))
