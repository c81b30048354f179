"""libpof's dense path (pof_dense_linear_filtsmooth, and pof_linear_filtsmooth
for uncompiled shapes with D >= 32) on the GPU against the NumPy float64
oracle on identical inputs.  The dense path runs the segmented chunked
schedule, restated as oracle.blocked.linear_filtsmooth_blocked(segmented=True)
with the same chunks; the expected values below are that schedule and the
reference scan (oracle.filtsmooth).  Tolerance: 1e-10 relative (normwise) on
means, on covariances compared as L L^T and on NLL / objectives / sigma^2;
float32 against float64 within the tolerance printed by the test."""

import numpy as np
import pytest
import torch

from oracle import blocked, filtsmooth as ofs, ivp as oivp, solver as osolver
from pof import _lib, parallel_filtsmooth as pfs
from pof.parallel_filtsmooth import _call
from pof.utils import MVNSqrt

pytestmark = pytest.mark.gpu

TOL = 1e-10


def T(x, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def N_(x):
    return x.detach().double().cpu().numpy()


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def covrel(a, b):
    A = a @ np.swapaxes(a, -1, -2)
    B = b @ np.swapaxes(b, -1, -2)
    return rel(A, B)


def _converged_problem(ivp, N, q, iters):
    ts = np.linspace(ivp.t0, ivp.tmax, N)
    states, info, st = osolver.solve(ivp, ts, q, init="constant", maxiters=iters, return_full=True)
    dom = osolver.linearize_at_previous_states(st, states[0])
    return st.x0, (st.F, st.QL), dom


def _random_problem(seed, n, D, d, with_R):
    rng = np.random.default_rng(seed)
    F = np.eye(D) + (0.3 / np.sqrt(D)) * rng.standard_normal((n, D, D))
    QL = np.tril((0.3 / np.sqrt(D)) * rng.standard_normal((n, D, D)))
    QL[:, np.arange(D), np.arange(D)] = 0.2 + 0.1 * rng.random((n, D))
    H = rng.standard_normal((n, d, D)) / np.sqrt(D)
    c = rng.standard_normal((n, d))
    R = None
    if with_R:
        R = np.tril(0.1 * rng.standard_normal((n, d, d)))
        R[:, np.arange(d), np.arange(d)] = 0.3
    m0 = rng.standard_normal(D)
    L0 = np.tril((0.2 / np.sqrt(D)) * rng.standard_normal((D, D))) + 0.5 * np.eye(D)
    return (m0, L0), (F, QL), (H, c, R)


def _chunk_plan(n, chunks):
    p = chunks if chunks > 0 else 64
    p = max(1, min(p, n))
    C0 = -(-n // p)
    return C0, -(-n // C0)


def _expected(x0, dtm, dom, C0, P):
    H, c, R = dom
    n, d, D = H.shape
    Rs = np.zeros((n, d, d)) if R is None else R
    (fm, fL), nll, fobj, ssq, _ = blocked.filter_blocked(x0, dtm, (H, c, Rs), C0=C0, Cs=(2,), segmented=True)
    (sm, sL), sobj = blocked.smoother_blocked(dtm, (fm, fL), C0=C0, Cs=(2,), segmented=True)
    return (fm, fL), (sm, sL), nll, fobj, sobj, ssq


def _gpu(which, x0, dtm, dom, chunks, per_step=True, dtype=torch.float64):
    F, QL = dtm
    H, c, R = dom
    if not per_step:
        F, QL = F[0], QL[0]
    x0t = MVNSqrt(T(x0[0], dtype), T(x0[1], dtype))
    dom_t = (T(H, dtype), T(c, dtype), None if R is None else T(R, dtype))
    out, nll, obj, ssq, scal = _call.filtsmooth(which, x0t, (T(F, dtype), T(QL, dtype)), dom_t, dense_chunks=chunks)
    torch.cuda.synchronize()
    return N_(out.mean), N_(out.chol), N_(scal)


SOLVER_CASES = {  # vdp_q3 with 5 chunks: C0 = 26, the last chunk 25 steps
    "logistic_q2": (lambda: oivp.logistic(r=3.0), 77, 2, 30),
    "vdp_q3": (lambda: oivp.vanderpol(stiffness_constant=1.0), 130, 3, 30),
    "rigid_q3": (lambda: oivp.rigid_body(), 64, 3, 20),
}


@pytest.mark.parametrize("chunks", [1, 5, 0])
@pytest.mark.parametrize("name", sorted(SOLVER_CASES))
def test_dense_path_on_solver_models(name, chunks):
    """Small-D models of converged IEKS iterations forced through the dense
    path: the segmented schedule's and the reference scan's results."""
    mk, N, q, its = SOLVER_CASES[name]
    x0, dtm, dom = _converged_problem(mk(), N, q, its)
    n = dom[0].shape[0]
    C0, P = _chunk_plan(n, chunks)
    m, L, sc = _gpu("filtsmooth", x0, dtm, dom, chunks, per_step=False)
    (fm, fL), (sm, sL), nll, fobj, sobj, ssq = _expected(x0, dtm, dom, C0, P)
    (rm, rL), rnll, robj, rssq = ofs.linear_filtsmooth(x0, dtm, dom)
    print("%s chunks=%d: means %.2e, LL^T %.2e, nll %.2e, obj %.2e; vs the reference scan: means %.2e"
          % (name, chunks, rel(m, sm), covrel(L, sL), abs(sc[0] - nll) / abs(nll), abs(sc[1] - sobj) / abs(sobj),
             rel(m, rm)))
    assert rel(m, sm) <= TOL and covrel(L, sL) <= TOL
    assert abs(sc[0] - nll) <= TOL * abs(nll)
    assert abs(sc[1] - sobj) <= TOL * max(abs(sobj), 1e-300) or abs(sc[1] - sobj) <= 1e-14
    assert abs(sc[3] - fobj) <= TOL * max(abs(fobj), 1e-300) or abs(sc[3] - fobj) <= 1e-14
    assert rel(m, rm) <= TOL and covrel(L, rL) <= TOL


@pytest.mark.parametrize("n,D,d,chunks,with_R,per_step", [
    (40, 48, 8, 8, False, True),
    (33, 64, 16, 4, True, False),
    (24, 96, 32, 6, False, False),
    (5, 160, 32, 2, True, True),
    (1, 40, 4, 0, False, True),
    (23, 40, 1, 4, False, True),
    (61, 36, 6, 9, True, True),
])
def test_dense_path_on_random_models(n, D, d, chunks, with_R, per_step):
    """Random dense models (D up to 160): filter + smoother, filter alone,
    smoother alone, against the segmented schedule."""
    x0, dtm, dom = _random_problem(n * 7 + D, n, D, d, with_R)
    F, QL = dtm
    if not per_step:
        F = np.broadcast_to(F[0], F.shape).copy()
        QL = np.broadcast_to(QL[0], QL.shape).copy()
        dtm = (F, QL)
    C0, P = _chunk_plan(n, chunks)
    (fm, fL), (sm, sL), nll, fobj, sobj, ssq = _expected(x0, dtm, dom, C0, P)
    m, L, sc = _gpu("filtsmooth", x0, dtm, dom, chunks, per_step)
    print("D=%d d=%d n=%d: means %.2e, LL^T %.2e, nll %.2e, ssq %.2e, fobj %.2e, sobj %.2e"
          % (D, d, n, rel(m, sm), covrel(L, sL), abs(sc[0] - nll) / abs(nll), abs(sc[2] - ssq) / abs(ssq),
             abs(sc[3] - fobj) / abs(fobj), abs(sc[1] - sobj) / abs(sobj)))
    assert rel(m, sm) <= TOL and covrel(L, sL) <= TOL
    for got, want in ((sc[0], nll), (sc[1], sobj), (sc[3], fobj)):
        assert abs(got - want) <= TOL * abs(want)
    # sigma^2 whitens with P11^{-T} (the reference's quirk, pof/utils.py:110-112):
    # for d >= 2 it depends on rounding-level sign choices inside tria, so it is
    # compared for d = 1 only (as in the small-D parity tests)
    assert np.isfinite(sc[2]) and sc[2] > 0
    if d == 1:
        assert abs(sc[2] - ssq) <= TOL * abs(ssq)
    mf, Lf, scf = _gpu("filter", x0, dtm, dom, chunks, per_step)
    assert rel(mf, fm) <= TOL and covrel(Lf, fL) <= TOL
    assert abs(scf[1] - fobj) <= TOL * abs(fobj)
    Fd, QLd = (T(F), T(QL)) if per_step else (T(F[0]), T(QL[0]))
    out, obj = _call.smoothing((Fd, QLd), MVNSqrt(T(mf), T(Lf)), dense_chunks=chunks)
    assert rel(N_(out.mean), sm) <= TOL and covrel(N_(out.chol), sL) <= TOL
    assert abs(float(obj) - sobj) <= TOL * abs(sobj)


def test_uncompiled_large_shape_takes_the_dense_path():
    """pof.parallel_filtsmooth at (D, d) = (48, 6), which no small-D table
    compiles: libpof's own entry points (filter + smoother, filter alone,
    smoother alone) run the dense path."""
    assert _lib.lib().pof_shape_supported(48, 6) == 0
    n, D, d = 30, 48, 6
    x0, dtm, dom = _random_problem(5, n, D, d, False)
    C0, P = _chunk_plan(n, 0)
    (fm, fL), (sm, sL), nll, fobj, sobj, ssq = _expected(x0, dtm, dom, C0, P)
    out, gnll, gobj, gssq = pfs.linear_filtsmooth(MVNSqrt(T(x0[0]), T(x0[1])), (T(dtm[0]), T(dtm[1])),
                                                  (T(dom[0]), T(dom[1]), None))
    assert rel(N_(out.mean), sm) <= TOL and covrel(N_(out.chol), sL) <= TOL
    assert abs(float(gnll) - nll) <= TOL * abs(nll) and abs(float(gobj) - sobj) <= TOL * abs(sobj)
    # the filter alone and the smoother alone through their own entry points
    fout, fnll, fobj_, _ = pfs.linear_noiseless_filtering(MVNSqrt(T(x0[0]), T(x0[1])), (T(dtm[0]), T(dtm[1])),
                                                          (T(dom[0]), T(dom[1]), None))
    assert rel(N_(fout.mean), fm) <= TOL and covrel(N_(fout.chol), fL) <= TOL
    assert abs(float(fobj_) - fobj) <= TOL * abs(fobj)
    sout, sobj_ = pfs.smoothing((T(dtm[0]), T(dtm[1])), MVNSqrt(T(fm), T(fL)))
    assert rel(N_(sout.mean), sm) <= TOL and covrel(N_(sout.chol), sL) <= TOL
    assert abs(float(sobj_) - sobj) <= TOL * abs(sobj)


def test_dense_path_at_d640():
    """The reaction-diffusion shape (D, d) = (640, 128): a few steps over two
    chunks against the segmented schedule."""
    n, D, d = 4, 640, 128
    x0, dtm, dom = _random_problem(640, n, D, d, False)
    C0, P = _chunk_plan(n, 2)
    (fm, fL), (sm, sL), nll, fobj, sobj, ssq = _expected(x0, dtm, dom, C0, P)
    m, L, sc = _gpu("filtsmooth", x0, dtm, dom, 2, per_step=True)
    print("D=640: means %.2e, LL^T %.2e, nll %.2e" % (rel(m, sm), covrel(L, sL), abs(sc[0] - nll) / abs(nll)))
    assert rel(m, sm) <= TOL and covrel(L, sL) <= TOL
    assert abs(sc[0] - nll) <= TOL * abs(nll)


@pytest.mark.parametrize("tf32", ["1", "0"])
@pytest.mark.parametrize("n,D,d", [(48, 64, 8), (12, 640, 128)])
def test_dense_float32_against_float64(monkeypatch, tf32, n, D, d):
    """The float32 dense pass (GEMMs on the tensor cores with 3xTF32
    products, or with POF_DENSE_TF32=0 on the FP32 pipe) against the float64
    one on the same model."""
    monkeypatch.setenv("POF_DENSE_TF32", tf32)
    x0, dtm, dom = _random_problem(32 + D, n, D, d, False)
    m64, L64, _ = _gpu("filtsmooth", x0, dtm, dom, 6)
    m32, L32, _ = _gpu("filtsmooth", x0, dtm, dom, 6, dtype=torch.float32)
    tol = 1e-4
    print("float32 dense (3xTF32 %s) vs float64, D=%d: means %.2e, LL^T %.2e (tolerance %.0e)"
          % (tf32, D, rel(m32, m64), covrel(L32, L64), tol))
    assert rel(m32, m64) <= tol and covrel(L32, L64) <= tol


def test_dense_deterministic():
    n, D, d = 20, 48, 8
    x0, dtm, dom = _random_problem(9, n, D, d, True)
    a = _gpu("filtsmooth", x0, dtm, dom, 4)
    b = _gpu("filtsmooth", x0, dtm, dom, 4)
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


# ---------------------------------------------------------------------------
# the reaction-diffusion FitzHugh-Nagumo field (pof.ivp.fhn_reaction_diffusion)
# ---------------------------------------------------------------------------

from pof import ivp as pivp, solver as psolver  # noqa: E402


@pytest.mark.parametrize("cells,q", [(2, 4), (4, 3), (64, 4)])
def test_rd_linearization_matches_oracle(cells, q):
    """pof_linearize of FIELD_FHN_RD (the dense path's kernel) against the
    oracle's EK1 (pof/observations.py:35-40 with the field's Jacobian) at
    random trajectories, including the (D, d) = (640, 128) shape."""
    ivp = oivp.fhn_reaction_diffusion(cells=cells)
    d = 2 * cells
    D = d * (q + 1)
    N = 9
    ts = np.linspace(0.0, 0.4, N)
    st = osolver.set_up_solver(ivp, ts, q)
    rng = np.random.default_rng(cells)
    means = rng.standard_normal((N, D))
    H, c, _ = osolver.linearize(st, means[1:])
    n = N - 1
    Hg = torch.empty((n, d, D), dtype=torch.float64, device="cuda")
    cg = torch.empty((n, d), dtype=torch.float64, device="cuda")
    p = T(np.array(ivp.params))
    rc = _lib.lib().pof_linearize(_lib.POF_F64, n, D, d, _lib.FIELDS["fhn_rd"], _lib.ptr(p), float(ts[1] - ts[0]),
                                  _lib.ptr(T(means)), _lib.ptr(Hg), _lib.ptr(cg), _lib.stream_handle())
    _lib.check(rc, "pof_linearize")
    torch.cuda.synchronize()
    print("cells=%d q=%d: H %.2e, c %.2e" % (cells, q, rel(N_(Hg), H), rel(N_(cg), c)))
    assert rel(N_(Hg), H) <= 1e-13 and rel(N_(cg), c) <= 1e-12


def _rd_problem(cells, q, N, tmax):
    ivp = oivp.fhn_reaction_diffusion(cells=cells, tmax=tmax)
    pv = pivp.fhn_reaction_diffusion(cells=cells, tmax=tmax)
    ts = np.linspace(0.0, tmax, N)
    return ivp, pv, ts


def test_rd_solve_matches_oracle():
    """The whole IEKS solve of the reaction-diffusion system at (D, d) =
    (32, 8) (4 cells, q = 3): pof.solver.solve runs the host-driven loop over
    pof_linearize and the dense filter/smoother; the oracle runs the same
    loop with the same chunked schedule (64 chunks)."""
    ivp, pv, ts = _rd_problem(4, 3, 97, 3.0)
    n = len(ts) - 1
    C0, P = _chunk_plan(n, 0)
    # uncalibrated: the calibration scales by sigma^2, which for d >= 2 is
    # rounding-defined (the reference's whiten quirk, pof/utils.py:110-112)
    (om, oL), oinfo = osolver.solve(ivp, ts, 3, init="constant", maxiters=200, calibrate=False,
                                    filtsmooth_fn=blocked.segmented_filtsmooth(C0, P))
    (gm, gL), ginfo = psolver.solve(f=pv.f, y0=pv.y0, ts=torch.as_tensor(ts), order=3, init="constant", maxiters=200,
                                    calibrate=False)
    gm, gL = N_(gm), N_(gL)
    # every ieks_step scales the factors by that iteration's sigma^2
    # (pof/step.py:33-45); compare L L^T / sigma^2
    gs, osq = float(ginfo["sigma_squared"]), float(oinfo["sigma_squared"])
    print("RD (32, 8): iterations %d (oracle %d), means %.2e, LL^T/sigma^2 %.2e, sigma^2 %.2e apart"
          % (int(ginfo["iterations"]), oinfo["iterations"], rel(gm, om), covrel(gL / gs ** 0.5, oL / osq ** 0.5),
             abs(gs - osq) / osq))
    assert int(ginfo["iterations"]) == oinfo["iterations"]
    assert int(ginfo["status"]) == 0
    assert rel(gm, om) <= TOL and covrel(gL / gs ** 0.5, oL / osq ** 0.5) <= TOL


def test_rd_mixed_precision_solve():
    """precision="mixed" on the reaction-diffusion system (host-driven float32
    phase over the dense path in float32, then the float64 loop): a float64
    IEKS fixed point within 1e-6 of the float64 solve, float32 iterations
    kept."""
    ivp, pv, ts = _rd_problem(4, 3, 97, 3.0)
    args = dict(f=pv.f, y0=pv.y0, ts=torch.as_tensor(ts), order=3, init="constant", maxiters=200)
    (m64, _), i64 = psolver.solve(**args)
    (mmx, _), imx = psolver.solve(precision="mixed", rtol_f32=1e-4, **args)
    err = rel(N_(mmx), N_(m64))
    print("RD mixed: float32 iterations %d, float64 %d (float64 alone %d), max rel error %.2e"
          % (int(imx["iterations_float32"]), int(imx["iterations"]), int(i64["iterations"]), err))
    assert int(imx["iterations_float32"]) >= 1
    assert err <= 1e-6


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-12), (torch.float32, 1e-4)])
def test_cluster_panels_match_single_cta_panels(monkeypatch, dtype, tol):
    """Panels of >= 256 columns factored by a 4-CTA cluster
    (k_tria_panel_cl) against one CTA per matrix (POF_DENSE_CLUSTER=0), at
    D = 160 (trias of 320 columns) and D = 640."""
    for n, D, d in ((20, 160, 16), (4, 640, 128)):
        x0, dtm, dom = _random_problem(3 * D, n, D, d, False)
        monkeypatch.setenv("POF_DENSE_CLUSTER", "1")
        m1, L1, s1 = _gpu("filtsmooth", x0, dtm, dom, 4, dtype=dtype)
        monkeypatch.setenv("POF_DENSE_CLUSTER", "0")
        m0, L0, s0 = _gpu("filtsmooth", x0, dtm, dom, 4, dtype=dtype)
        print("cluster vs single-CTA panels, D=%d %s: means %.2e, LL^T %.2e"
              % (D, dtype, rel(m1, m0), covrel(L1, L0)))
        assert rel(m1, m0) <= tol and covrel(L1, L0) <= tol
        assert abs(s1[0] - s0[0]) <= tol * abs(s0[0])
