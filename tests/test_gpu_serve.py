"""Continuous batching (pof_server_*, pof.serve): requests of several shapes
submitted while others iterate; every result bit-identical to the same
request served alone, and equal to the batched solve with the request's
chunk length; admission under a small memory budget."""

import numpy as np
import pytest
import torch

from oracle import blocked as oblocked, ivp as oivp, solver as osolver
from pof import batch as pbatch, serve

pytestmark = pytest.mark.gpu

# (field, params, y0, t1, N, q, rtol)
REQUESTS = [
    ("logistic", (1.0,), [0.01], 10.0, 200, 3, 1e-6),
    ("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], 7.0, 600, 3, 1e-6),
    ("vanderpol", (1.0,), [2.0, 0.0], 6.3, 128, 2, 1e-4),
    ("logistic", (1.5,), [0.02], 10.0, 2100, 4, 1e-4),
    ("fhn_classic", (0.2, 0.2, 3.0), [-1.0, 1.0], 5.0, 120, 3, 1e-6),
    ("vanderpol", (1.2,), [1.9, 0.1], 5.0, 257, 2, 1e-6),
    ("lotkavolterra", (1.3, 0.9, 2.8, 1.1), [1.2, 0.8], 5.0, 300, 3, 1e-4),
    ("fitzhughnagumo", (0.7, 0.8, 0.08, 0.5), [1.0, 1.0], 20.0, 90, 3, 1e-6),
]


def _submit(srv, r):
    nm, p, y0, t1, N, q, rtol = r
    return srv.submit(nm, p, y0, np.linspace(0.0, t1, N), q, rtol=rtol, maxiters=1000)


def _serve_mix(reqs, max_points=1 << 16, max_requests=64, stagger=3):
    """Submit reqs one by one, `stagger` ticks apart (later ones join while
    earlier ones iterate), then run until every request has finished."""
    srv = serve.Server(max_requests=max_requests, max_points=max_points)
    rids = []
    for r in reqs:
        rids.append(_submit(srv, r))
        for _ in range(stagger):
            srv.tick()
    guard = 0
    while srv.busy():
        srv.tick()
        guard += 1
        assert guard < 20000
    out = [srv.result(rid) for rid in rids]
    srv.close()
    return out


def _same(a, b):
    (ma, La), ia = a
    (mb, Lb), ib = b
    assert torch.equal(ma, mb) and torch.equal(La, Lb)
    for k in ("iterations", "nll", "obj", "sigma_squared"):
        assert float(ia[k]) == float(ib[k]), k


def test_served_result_same_alone_and_in_the_mix():
    mix = _serve_mix(REQUESTS)
    rev = _serve_mix(REQUESTS[::-1], stagger=1)
    for i, r in enumerate(REQUESTS):
        alone = _serve_mix([r])[0]
        _same(mix[i], alone)
        _same(mix[i], rev[len(REQUESTS) - 1 - i])


def test_served_equals_batched_solve():
    """A served request with the reference's tolerance is the batched solve
    of that problem with its chunk length, bit for bit."""
    mix = _serve_mix(REQUESTS)
    for i, (nm, p, y0, t1, N, q, rtol) in enumerate(REQUESTS):
        n = N - 1
        c0 = 4
        while c0 < 64 and c0 * 2 * 256 <= n:
            c0 *= 2
        (gm, gL), ginfo = mix[i]
        if rtol == 1e-6:  # the batched solve uses the reference's crit (rtol 1e-6)
            res = pbatch.solve_batch([(nm, p, y0, np.linspace(0.0, t1, N))], order=q, maxiters=1000, C0=c0, Cg=2)
            (bm, bL), binfo = res.problem(0)
            assert torch.equal(gm, bm) and torch.equal(gL, bL), nm


@pytest.mark.parametrize("i", [0, 2, 3])
def test_served_request_tolerance_matches_oracle(i):
    """The oracle's IEKS with the request's tolerance: the same iteration
    count, means within 1e-10 or 10x the spread to the oracle run with the
    served schedule (oracle.blocked.segmented_filtsmooth)."""
    nm, p, y0, t1, N, q, rtol = REQUESTS[i]
    (gm, _), ginfo = _serve_mix([REQUESTS[i]])[0]
    ts = np.linspace(0.0, t1, N)
    o = {"logistic": lambda: oivp.logistic(tmax=t1, y0=y0, r=p[0]),
         "vanderpol": lambda: oivp.vanderpol(tmax=t1, y0=y0, stiffness_constant=p[0])}[nm]()
    (om, _), oinfo = osolver.solve(o, ts, q, init="constant", maxiters=1000, rtol=rtol)
    n = N - 1
    c0 = 4
    while c0 < 64 and c0 * 2 * 256 <= n:
        c0 *= 2
    (sm, _), _ = osolver.solve(o, ts, q, init="constant", maxiters=1000, rtol=rtol,
                               filtsmooth_fn=oblocked.segmented_filtsmooth(c0, 2))
    assert int(ginfo["iterations"]) == oinfo["iterations"]
    spread = np.abs(sm - om).max() / np.abs(om).max()
    assert np.abs(gm.cpu().numpy() - om).max() / np.abs(om).max() <= max(1e-10, 10 * spread)


def test_admission_waits_for_memory():
    """An engine with room for about two requests at a time: the rest queue,
    are admitted as earlier ones finish, and give the same results."""
    reqs = [REQUESTS[0], REQUESTS[1], REQUESTS[4], REQUESTS[5]]
    tight = _serve_mix(reqs, max_points=700, max_requests=2, stagger=0)
    for i, r in enumerate(reqs):
        _same(tight[i], _serve_mix([r])[0])


# well-conditioned requests (one IEKS fixed point each) for the float32 + float64 form
MIXED_REQUESTS = [
    ("vanderpol", (1.0,), [2.0, 0.0], 6.3, 600, 3, 1e-6),
    ("logistic", (1.0,), [0.01], 10.0, 300, 3, 1e-6),
    ("vanderpol", (1.2,), [1.9, 0.1], 5.0, 1100, 4, 1e-6),
]


def _serve_mixed(reqs, stagger=2):
    srv = serve.Server(max_requests=16, max_points=1 << 15, precision="mixed")
    rids = []
    for r in reqs:
        nm, p, y0, t1, N, q, rtol = r
        rids.append(srv.submit(nm, p, y0, np.linspace(0.0, t1, N), q, rtol=rtol, maxiters=1000))
        for _ in range(stagger):
            srv.tick()
    guard = 0
    while srv.busy():
        srv.tick()
        guard += 1
        assert guard < 20000
    out = [srv.result(rid) for rid in rids]
    srv.close()
    return out


def test_served_mixed_precision():
    """The served float32 + float64-polish form: each request runs float32
    IEKS iterations, then float64 ones, in the same ticks as the others.
    Its result is the batched mixed solve of that problem with its chunk
    length, bit for bit, alone and in the mix (float32 iterations and their
    count included), and within 1e-6 of the served float64 result."""
    mix = _serve_mixed(MIXED_REQUESTS)
    f64 = _serve_mix(MIXED_REQUESTS)
    for i, r in enumerate(MIXED_REQUESTS):
        nm, p, y0, t1, N, q, rtol = r
        (gm, gL), gi = mix[i]
        assert gi["status"] == "converged" and int(gi["iterations_float32"]) > 0, (nm, gi)
        alone = _serve_mixed([r])[0]
        assert torch.equal(gm, alone[0][0]) and torch.equal(gL, alone[0][1])
        assert int(gi["iterations_float32"]) == int(alone[1]["iterations_float32"])
        n = N - 1
        c0 = 4
        while c0 < 64 and c0 * 2 * 256 <= n:
            c0 *= 2
        res = pbatch.solve_batch([(nm, p, y0, np.linspace(0.0, t1, N))], order=q, maxiters=1000, C0=c0, Cg=2,
                                 precision="mixed")
        (bm, bL), bi = res.problem(0)
        assert torch.equal(gm, bm) and torch.equal(gL, bL), nm
        assert int(gi["iterations"]) == int(bi["iterations"])
        assert int(gi["iterations_float32"]) == int(bi["iterations_float32"])
        (fm, _), fi = f64[i]
        err = float((gm - fm).abs().max() / fm.abs().max())
        print("[served mixed %s] float32 %d + float64 %d iterations (float64 alone %d), %.3g from float64" % (
            nm, int(gi["iterations_float32"]), int(gi["iterations"]), int(fi["iterations"]), err))
        assert err <= 1e-6


def test_served_dense_request_same_as_alone():
    """A reaction-diffusion request (a field of the dense path) is served by
    the dense lane -- its own IEKS loop on its own stream in a worker thread
    -- while small-D requests run in the engines; its result equals
    pof.solver.solve of the same request alone, bit for bit."""
    from pof import ivp as pivp, solver as psolver

    cells, q, N = 4, 3, 97
    pv = pivp.fhn_reaction_diffusion(cells=cells, tmax=3.0)
    ts = np.linspace(0.0, 3.0, N)
    params = (0.2, 0.2, 3.0, 0.5, 0.05)
    srv = serve.Server(max_requests=8, max_points=1 << 16)
    small = [srv.submit("logistic", (3.0,), [0.01], np.linspace(0.0, 10.0, n), 3) for n in (300, 900, 2000)]
    rid = srv.submit("fhn_rd", params, pv.y0.numpy(), ts, q, rtol=1e-6, maxiters=200)
    while srv.busy():
        srv.tick()
    (m, L), info = srv.result(rid)
    (m1, L1), info1 = psolver.solve(f=pv.f, y0=pv.y0, ts=torch.as_tensor(ts), order=q, init="constant",
                                    maxiters=200)
    print("served RD: status %s, iterations %d (alone %d)" % (info["status"], int(info["iterations"]),
                                                               int(info1["iterations"])))
    assert info["status"] == "converged" and int(info["iterations"]) == int(info1["iterations"])
    assert torch.equal(m.cpu(), m1.cpu()) and torch.equal(L.cpu(), L1.cpu())
    for r in small:
        assert srv.result(r)[1]["status"] == "converged"
    srv.close()
