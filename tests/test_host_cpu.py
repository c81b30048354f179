"""The torch host code of `pof` against the oracle, on CPU tensors.

Everything here runs in the drop-in package on the GPU path too: the
linear-algebra helpers of pof/utils.py, the convergence criterion, the
sequential one-step predict/update used by the initial trajectories, the
initial trajectories themselves ("prior" is the default `init` of
`pof.solver.solve`), the EK1 / EK0 / regularized linearizations of user
vector fields (torch.func.jacfwd), and the element-level operators of the
reference's parallel filter and smoother.  torch runs the same operations on
CPU and CUDA tensors, so these are checked here on the CPU.
"""

import numpy as np
import pytest
import torch

from oracle import core as oc, filtsmooth as ofs, ivp as oivp, solver as osolver
from pof import convergence_criteria as pcc, initialization as pinit, ivp as pivp, observations as pobs
from pof import transitions as ptr, utils as pu
from pof.sequential_filtsmooth.filter import _sqrt_predict, _sqrt_update
from pof.utils import MVNSqrt

CPU = torch.device("cpu")


def T(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64)


def lower(rng, *shape):
    return np.tril(rng.standard_normal(shape)) + 3.0 * np.eye(shape[-1])


def gram(L):
    return L @ np.swapaxes(L, -1, -2)


@pytest.fixture
def rng():
    return np.random.default_rng(20261204)


def test_tria_is_lapack_qr(rng):
    A = rng.standard_normal((7, 6, 13))
    L = pu.tria(T(A)).numpy()
    assert np.allclose(np.triu(L, 1), 0.0)
    assert np.allclose(L, oc.tria(A), rtol=1e-12, atol=1e-12)  # same signs, not just the same L L^T
    assert np.allclose(gram(L), gram(A), rtol=1e-12, atol=1e-12)


def test_whiten_solves_with_the_transpose(rng):
    """whiten(m, L) = L^-T m (the reference's solve_triangular(L.T, m) with
    lower=False), not L^-1 m."""
    L = lower(rng, 5, 4, 4)
    m = rng.standard_normal((5, 4))
    w = pu.whiten(T(m), T(L)).numpy()
    assert np.allclose(w, oc.whiten(m, L), rtol=1e-13, atol=1e-13)
    assert np.allclose(np.einsum("kji,kj->ki", L, w), m, rtol=1e-12, atol=1e-12)
    assert not np.allclose(w, np.linalg.solve(L, m[..., None])[..., 0])


def test_loglikelihood_objective_and_helpers(rng):
    L = lower(rng, 6, 3, 3)
    x = rng.standard_normal((6, 3))
    assert np.allclose(pu.mvn_loglikelihood(T(x), T(L)).numpy(), oc.mvn_loglikelihood(x, L), rtol=1e-13)
    F = rng.standard_normal((6, 3, 3))
    QL = lower(rng, 6, 3, 3)
    mn, m = rng.standard_normal((6, 3)), rng.standard_normal((6, 3))
    a = pu.objective_function_value(T(mn), T(m), (T(F), T(QL))).numpy()
    assert np.allclose(a, oc.objective_function_value(mn, m, F, QL), rtol=1e-13)
    z = rng.standard_normal((3, 2))
    assert np.array_equal(pu.append_zeros_along_new_axis(T(z), 4).numpy(), oc.append_zeros_along_new_axis(z, 4))
    A = rng.standard_normal((2, 3))
    g = pu.gmul_stack(T(A), MVNSqrt(T(m), T(L)))
    assert np.allclose(g.mean.numpy(), m @ A.T) and np.allclose(g.chol.numpy(), A @ L)


@pytest.mark.parametrize("case", range(12))
def test_crit_matches_oracle(rng, case):
    means_old = rng.standard_normal((9, 4))
    means = means_old + (0.0 if case % 3 == 0 else 10.0 ** -(4 + 3 * (case % 4))) * rng.standard_normal((9, 4))
    obj_old = float(rng.uniform(1, 1e3))
    obj = obj_old * (1 + (1e-7 if case % 2 else 1e-3))
    nll, nll_old = float(rng.standard_normal()), float(rng.standard_normal())
    if case == 5:
        nll = float("nan")
    if case == 7:
        obj = float("nan")
    kw = {} if case < 8 else {"rtol": 1e-2, "atol": 1e-2}
    want = osolver.crit(obj, obj_old, nll, nll_old, means, means_old, **kw)
    got = pcc.crit(obj, obj_old, nll, nll_old, MVNSqrt(T(means), None), MVNSqrt(T(means_old), None), **kw)
    assert bool(got) == bool(want)


@pytest.mark.parametrize("with_R", [False, True])
def test_sqrt_predict_and_update_match_oracle(rng, with_R):
    D, d, B = 6, 2, 5
    F = rng.standard_normal((B, D, D))
    QL = lower(rng, B, D, D)
    m = rng.standard_normal((B, D))
    L = lower(rng, B, D, D)
    pm, pL = _sqrt_predict(T(F), T(QL), MVNSqrt(T(m), T(L)))
    om, oL = ofs.sqrt_predict(F, QL, m, L)
    assert np.allclose(pm.numpy(), om, rtol=1e-13) and np.allclose(gram(pL.numpy()), gram(oL), rtol=1e-12)
    for k in range(B):  # the torch helper is one step at a time
        H = rng.standard_normal((d, D))
        c = rng.standard_normal(d)
        R = lower(rng, d, d) if with_R else np.zeros((d, d))
        (um, uL), ell, ssq = _sqrt_update(T(H), T(R), T(c), MVNSqrt(T(om[k]), T(oL[k])))
        (vm, vL), vell, vssq = ofs.sqrt_update(H, R, c, om[k], oL[k])
        assert np.allclose(um.numpy(), vm, rtol=1e-11, atol=1e-12)
        assert np.allclose(gram(uL.numpy()), gram(vL), rtol=1e-11, atol=1e-12)
        assert np.isclose(float(ell), vell, rtol=1e-12) and np.isclose(float(ssq), vssq, rtol=1e-11)


CASES = [("logistic", {"r": 3.0}, 10.0, 2), ("fhn_classic", {}, 100.0, 3), ("lotkavolterra", {}, 7.0, 4),
         ("vanderpol", {"stiffness_constant": 1.0}, 6.3, 3)]


@pytest.mark.parametrize("name,kw,t1,q", CASES)
def test_constant_and_prior_init_match_oracle(name, kw, t1, q):
    """The "constant" trajectory, and the default "prior" one with the
    reference's quirks: transitions at step sizes ts[1:] (absolute times),
    not preconditioned, not scaled by PI."""
    p, o = getattr(pivp, name)(**kw), getattr(oivp, name)(**kw)
    ts = np.linspace(0.0, t1, 40)
    c = pinit.constant_init(y0=p.y0, order=q, ts=ts, f=p.f, device=CPU)
    om, oL = osolver.constant_init(o, q, ts)
    assert np.allclose(c.mean.numpy(), om, rtol=1e-14) and np.array_equal(c.chol.numpy(), oL)
    pr = pinit.prior_init(f=p.f, y0=p.y0, order=q, ts=ts, device=CPU)
    om, oL = osolver.prior_init(o, q, ts)
    scale = np.abs(om).max(axis=0) + 1e-300
    assert np.allclose(pr.mean.numpy() / scale, om / scale, rtol=1e-12, atol=1e-12)
    G, oG = gram(pr.chol.numpy()), gram(oL)
    assert np.allclose(G, oG, rtol=1e-10, atol=1e-10 * np.abs(oG).max())


@pytest.mark.parametrize("name,kw,t1,q", CASES)
def test_ek1_linearization_of_a_user_field_matches_oracle(rng, name, kw, t1, q):
    """torch.func.jacfwd EK1 of the residual E1 P x - f(E0 P x) at a batch of
    states (pof/observations.py:35-40) == the oracle's analytic Jacobians."""
    p, o = getattr(pivp, name)(**kw), getattr(oivp, name)(**kw)
    ts = np.linspace(0.0, t1, 33)
    st = osolver.set_up_solver(o, ts, q)
    d = st.d
    iwp = ptr.IWP(wiener_process_dimension=d, num_derivatives=q)
    P, _ = ptr.nordsieck_preconditioner(iwp, ts[1] - ts[0], device=CPU)
    E0 = ptr.projection_matrix(iwp, 0, device=CPU) @ P
    E1 = ptr.projection_matrix(iwp, 1, device=CPU) @ P
    assert np.allclose(E0.numpy(), st.E0, rtol=1e-15) and np.allclose(E1.numpy(), st.E1, rtol=1e-15)

    def om_fn(x):
        return E1 @ x - p.f(None, E0 @ x)

    means, _ = osolver.get_initial_trajectory(st, "constant")
    means = means[1:] * (1 + 0.1 * rng.standard_normal(means[1:].shape))
    D = means.shape[1]
    H, b, R = pobs.linearize(om_fn, MVNSqrt(T(means), torch.zeros(len(means), D, D, dtype=torch.float64)))
    oH, oc_, oR = osolver.linearize(st, means)
    assert np.allclose(H.numpy(), oH, rtol=1e-12, atol=1e-12 * np.abs(oH).max())
    assert np.allclose(b.numpy(), oc_, rtol=1e-10, atol=1e-10 * np.abs(oc_).max())
    assert np.array_equal(R.numpy(), oR)


def test_ek0_and_regularized_linearizations(rng):
    """EK0: H = E1, b = f(m) - E1 m (pof/observations.py:52-61); the
    Levenberg-Marquardt form stacks the EK1 rows on (I, -m) with noise
    chol blockdiag(0, I / sqrt(l)) (pof/observations.py:64-83)."""
    p = pivp.lotkavolterra()
    q, d = 3, 2
    D = d * (q + 1)
    iwp = ptr.IWP(wiener_process_dimension=d, num_derivatives=q)
    E0 = ptr.projection_matrix(iwp, 0, device=CPU)
    E1 = ptr.projection_matrix(iwp, 1, device=CPU)

    def om_fn(x):
        return E1 @ x - p.f(None, E0 @ x)

    m = T(rng.uniform(0.5, 1.5, D))
    x = MVNSqrt(m, torch.eye(D, dtype=torch.float64))
    H0, b0, R0 = pobs.linearize_ek0(om_fn, x)
    assert torch.equal(H0, E1) and torch.allclose(b0, om_fn(m) - E1 @ m) and not R0.any()
    H, b, R = pobs.linearize(om_fn, x)
    lam = 4.0
    Hr, br, Rr = pobs.linearize_regularized(om_fn, x, lam)
    assert Hr.shape == (d + D, D) and br.shape == (d + D,) and Rr.shape == (d + D, d + D)
    assert torch.allclose(Hr[:d], H) and torch.equal(Hr[d:], torch.eye(D, dtype=torch.float64))
    assert torch.allclose(br[:d], om_fn(m)) and torch.equal(br[d:], -m)
    assert not Rr[:d].any() and not Rr[:, :d].any()
    assert torch.allclose(Rr[d:, d:], torch.eye(D, dtype=torch.float64) / lam**0.5)
    # b of the EK1 rows is f(m) - H m there, f(m) in the regularized form (the reference's full_b = [res, -m])
    assert torch.allclose(b, om_fn(m) - H @ m)


def _filter_elements(rng, B, D, d):
    """B filter elements of random models with the reference's element
    construction (the oracle's get_element, filter.py:50-81)."""
    F = rng.standard_normal((B, D, D)) / np.sqrt(D)
    QL = lower(rng, B, D, D) * 0.3
    H = rng.standard_normal((B, d, D))
    c = rng.standard_normal((B, d))
    R = np.zeros((B, d, d))
    return ofs.get_element(F, QL, H, c, R, np.zeros((B, D)), np.zeros((B, D, D)))


def _same_element(a, b, tol):
    A, bb, U, eta, Z = (x.numpy() if isinstance(x, torch.Tensor) else x for x in a)
    oA, ob, oU, oeta, oZ = b
    for x, y in ((A, oA), (bb, ob), (eta, oeta), (gram(U), gram(oU)), (gram(Z), gram(oZ))):
        assert np.allclose(x, y, rtol=tol, atol=tol * max(np.abs(y).max(), 1.0))


def test_filtering_operator_matches_oracle_and_is_associative(rng):
    from pof.parallel_filtsmooth.filter import sqrt_filtering_operator

    B, D, d = 6, 6, 2
    e1, e2, e3 = (_filter_elements(rng, B, D, d) for _ in range(3))
    t = lambda e: tuple(T(x) for x in e)  # noqa: E731
    got = sqrt_filtering_operator(t(e1), t(e2))
    _same_element(got, ofs.sqrt_filtering_operator(e1, e2), 1e-11)
    left = sqrt_filtering_operator(sqrt_filtering_operator(t(e1), t(e2)), t(e3))
    right = sqrt_filtering_operator(t(e1), sqrt_filtering_operator(t(e2), t(e3)))
    _same_element(left, tuple(x.numpy() for x in right), 1e-9)


def test_smoother_elements_and_operator_match_oracle(rng):
    from pof.parallel_filtsmooth.smoother import get_elements, sqrt_smoothing_operator

    N, D = 9, 5
    F = rng.standard_normal((N - 1, D, D)) / np.sqrt(D)
    QL = lower(rng, N - 1, D, D) * 0.3
    ms = rng.standard_normal((N, D))
    Ls = lower(rng, N, D, D)
    g, E, L = get_elements((T(F), T(QL)), MVNSqrt(T(ms), T(Ls)))
    og, oE, oL = ofs.get_smoother_elements((F, QL), (ms, Ls))
    assert np.allclose(g.numpy(), og, rtol=1e-11, atol=1e-11) and np.allclose(E.numpy(), oE, rtol=1e-11, atol=1e-11)
    assert np.allclose(gram(L.numpy()), gram(oL), rtol=1e-11, atol=1e-11)
    a = (g[1:], E[1:], L[1:])
    b = (g[:-1], E[:-1], L[:-1])
    cg, cE, cD = sqrt_smoothing_operator(a, b)
    og, oE, oD = ofs.sqrt_smoothing_operator((og[1:], oE[1:], oL[1:]), (og[:-1], oE[:-1], oL[:-1]))
    assert np.allclose(cg.numpy(), og, rtol=1e-11, atol=1e-11) and np.allclose(cE.numpy(), oE, rtol=1e-11, atol=1e-11)
    assert np.allclose(gram(cD.numpy()), gram(oD), rtol=1e-11, atol=1e-11)


def test_utils_linearize_is_the_first_order_model():
    f = lambda x: torch.stack([x[0] * x[1], torch.sin(x[0]) + x[1] ** 3])  # noqa: E731
    x = torch.tensor([0.3, -1.2], dtype=torch.float64)
    A, b = pu.linearize(f, x)
    J = torch.tensor([[x[1], x[0]], [torch.cos(x[0]), 3 * x[1] ** 2]], dtype=torch.float64)
    assert torch.allclose(A, J) and torch.allclose(b, f(x) - J @ x)
    assert torch.allclose(pu.AffineModel(A, b)(x), f(x))


@pytest.mark.parametrize("multiplier", [1.0, 0.25])
def test_cholesky_update_many(rng, multiplier):
    """L' L'^T = L L^T + multiplier sum_k v_k v_k^T, L' lower-triangular."""
    n = 5
    L = lower(rng, n, n)
    V = rng.standard_normal((3, n))
    out = pu.cholesky_update_many(T(L), T(V), multiplier).numpy()
    assert np.array_equal(out, np.tril(out))
    assert np.allclose(gram(out), gram(L) + multiplier * V.T @ V, rtol=1e-12, atol=1e-12)


def test_trajectory_linearizers_of_the_iterators(rng):
    """lom / lom_reg (pof/iterators.py:14-17) stack the one-state
    linearizations over a trajectory."""
    from pof import iterators as pit

    E1 = T(np.kron(np.eye(2), np.eye(1, 3, 1)))
    E0 = T(np.kron(np.eye(2), np.eye(1, 3, 0)))
    p = pivp.lotkavolterra()
    om = pobs.NonlinearModel(lambda x: E1 @ x - p.f(None, E0 @ x))
    traj = MVNSqrt(T(rng.uniform(0.5, 1.5, (4, 6))), torch.zeros(4, 6, 6, dtype=torch.float64))
    H, b, R = pit.lom(om, traj)
    Hr, br, Rr = pit.lom_reg(om, traj, 2.0)
    for k in range(4):
        x = MVNSqrt(traj.mean[k], traj.chol[k])
        h, bb, r = pobs.linearize(om, x)
        assert torch.allclose(H[k], h) and torch.allclose(b[k], bb) and torch.equal(R[k], r)
        h, bb, r = pobs.linearize_regularized(om, x, 2.0)
        assert torch.allclose(Hr[k], h) and torch.allclose(br[k], bb) and torch.equal(Rr[k], r)


def test_uncertain_and_classic_inits():
    """uncertain_init (initialization.py:25-39): mean [y0, f(y0), 0, ...] per
    dimension, chol sqrt(var) except 0 on each dimension's first two
    derivatives; classic_to_init (:59-72): [y, f(y), 0, ...] rows, chol 0."""
    p = pivp.lotkavolterra()
    q, d = 3, 2
    x = pinit.uncertain_init(p.f, p.y0, q, var=4.0, device=CPU)
    f0 = p.f(None, p.y0)
    want = torch.zeros(d, q + 1, dtype=torch.float64)
    want[:, 0], want[:, 1] = p.y0, f0
    assert torch.allclose(x.mean, want.reshape(-1))
    diag = torch.full((d, q + 1), 2.0, dtype=torch.float64)
    diag[:, :2] = 0.0
    assert torch.equal(x.chol, torch.diag(diag.reshape(-1)))
    ys = torch.tensor([[1.0, 1.0], [0.5, 2.0], [3.0, 0.1]], dtype=torch.float64)
    c = pinit.classic_to_init(ys=ys, order=q, f=p.f)
    for k in range(3):
        row = torch.zeros(d, q + 1, dtype=torch.float64)
        row[:, 0], row[:, 1] = ys[k], p.f(None, ys[k])
        assert torch.allclose(c.mean[k], row.reshape(-1))
    assert not c.chol.any()


def test_updated_prior_init_matches_oracle():
    """updated_prior_init (initialization.py:92-100): the one-step prior
    predictions from x0, each updated by the noiseless EK1 observation at
    its own mean."""
    q = 2
    p, o = pivp.vanderpol(stiffness_constant=1.0), oivp.vanderpol(stiffness_constant=1.0)
    ts = np.linspace(0.0, 6.3, 12)
    st = osolver.set_up_solver(o, ts, q)
    iwp = ptr.IWP(wiener_process_dimension=2, num_derivatives=q)
    P, PI = ptr.nordsieck_preconditioner(iwp, ts[1] - ts[0], device=CPU)
    E0 = ptr.projection_matrix(iwp, 0, device=CPU) @ P
    E1 = ptr.projection_matrix(iwp, 1, device=CPU) @ P
    om = pobs.NonlinearModel(lambda x: E1 @ x - p.f(None, E0 @ x))
    x0 = MVNSqrt(T(st.x0[0]), T(st.x0[1]) + T(0.1 * np.eye(6)))
    dtm = (T(st.F), T(st.QL))
    got = pinit.updated_prior_init(x0=x0, dtm=dtm, om=om)
    pm, pL = ofs.sqrt_predict(st.F, st.QL, np.broadcast_to(_np_(x0.mean), (len(ts) - 1, 6)),
                              np.broadcast_to(_np_(x0.chol), (len(ts) - 1, 6, 6)))
    pm = np.concatenate([_np_(x0.mean)[None], pm])
    pL = np.concatenate([_np_(x0.chol)[None], pL])
    H, c, R = osolver.linearize(st, pm)
    for k in range(len(ts)):
        (m, L), _, _ = ofs.sqrt_update(H[k], R[k], c[k], pm[k], pL[k])
        assert np.allclose(got.mean[k].numpy(), m, rtol=1e-10, atol=1e-12)
        assert np.allclose(gram(got.chol[k].numpy()), gram(L), rtol=1e-9, atol=1e-12)


def _np_(t):
    return t.detach().numpy()


FIELDS = [("logistic", {}), ("logistic", {"r": 3.0}), ("lotkavolterra", {}), ("vanderpol", {}),
          ("fitzhughnagumo", {}), ("fhn_classic", {}), ("rober", {}), ("rigid_body", {}), ("seir", {}),
          ("threebody", {}), ("henonheiles", {}), ("fhn_reaction_diffusion", {"cells": 6}),
          ("fhn_reaction_diffusion", {"cells": 2, "kv": 0.7, "kw": 0.1})]


@pytest.mark.parametrize("name,kw", FIELDS)
def test_builtin_fields_match_the_oracle(rng, name, kw):
    """Every pof.ivp field (torch) against the oracle's restatement of
    pof/ivp.py: values and Jacobians (torch.func.jacfwd against the oracle's
    forward-mode Jacobian) at perturbed initial values, and the same y0,
    time span and parameters."""
    p, o = getattr(pivp, name)(**kw), getattr(oivp, name)(**kw)
    assert np.array_equal(p.y0.numpy(), o.y0) and (p.t0, p.tmax) == (o.t0, o.tmax)
    assert p.f.pof_field == (o.name, tuple(float(x) for x in o.params))
    for _ in range(3):
        y = o.y0 * (1 + 0.1 * rng.standard_normal(o.y0.shape)) + 0.01 * rng.standard_normal(o.y0.shape)
        fy = p.f(None, T(y)).numpy()
        assert np.allclose(fy, o.f(None, y), rtol=1e-13, atol=1e-13 * max(1.0, np.abs(fy).max()))
        J = torch.func.jacfwd(lambda yy: p.f(None, yy))(T(y)).numpy()
        assert np.allclose(J, o.jac(y), rtol=1e-12, atol=1e-12 * max(1.0, np.abs(J).max()))


@pytest.mark.parametrize("cells", [1, 2, 5])
def test_reaction_diffusion_forms_agree(rng, cells):
    """The oracle's reaction-diffusion system in its three forms -- the
    Taylor components (used for Taylor-mode initial values), the array field
    and its analytic Jacobian -- agree with each other and with the torch
    field's torch.func.jacfwd, periodic neighbours included (one and two
    cells: the neighbours coincide and their couplings add up)."""
    from oracle import taylor

    o = oivp.fhn_reaction_diffusion(cells=cells, kv=0.3, kw=0.07)
    p = pivp.fhn_reaction_diffusion(cells=cells, kv=0.3, kw=0.07)
    for _ in range(3):
        y = o.y0 + 0.3 * rng.standard_normal(o.y0.shape)
        f_arr = o.f(None, y)
        f_cmp = np.asarray(taylor.evaluate(o.components, y), dtype=np.float64)
        assert np.allclose(f_arr, f_cmp, rtol=1e-14, atol=1e-14)
        J_arr = o.jac(y)
        J_cmp = taylor.jacobian(o.components, y)
        assert np.allclose(J_arr, J_cmp, rtol=1e-13, atol=1e-13)
        J_t = torch.func.jacfwd(lambda yy: p.f(None, yy))(T(y)).numpy()
        assert np.allclose(J_t, J_arr, rtol=1e-13, atol=1e-13)
