"""Batched solves (pof_ieks_solve_batch) against the float64 oracle, problem
by problem, and the batch invariants: a problem's result does not depend on
the other problems of the batch, on their order, on re-planning or on the
CUDA-graph replay."""

import os

import numpy as np
import pytest
import torch

from oracle import blocked as oblocked, ivp as oivp, solver as osolver
from oracle.scan import sequential_scan
from pof import batch as pbatch, ivp as pivp, solver as psolver

pytestmark = pytest.mark.gpu

TOL = 1e-10


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def covrel(a, b):
    A = a @ np.swapaxes(a, -1, -2)
    B = b @ np.swapaxes(b, -1, -2)
    return rel(A, B)


def close(x, ref, alt):
    return abs(float(x) - ref) <= max(TOL * abs(ref), 10.0 * abs(ref - alt), 1e-300)


def oracle_ivp(name, params, y0, t0, t1):
    if name == "logistic":
        return oivp.logistic(t0=t0, tmax=t1, y0=y0, r=params[0])
    if name == "lotkavolterra":
        return oivp.lotkavolterra(t0=t0, tmax=t1, y0=y0, p=params)
    if name == "vanderpol":
        return oivp.vanderpol(t0=t0, tmax=t1, y0=y0, stiffness_constant=params[0])
    if name == "fhn_classic":
        a, b, c = params
        return oivp.fhn_classic(t0=t0, tmax=t1, y0=y0, a=a, b=b, c=c)
    if name == "fitzhughnagumo":
        return oivp.fitzhughnagumo(t0=t0, tmax=t1, y0=y0, p=params)
    raise ValueError(name)


# (field, params, y0, t0, t1, N); one batch per dimension, fields mixed
BATCH_D1 = [
    ("logistic", (1.0,), [0.01], 0.0, 10.0, 200),
    ("logistic", (1.5,), [0.02], 0.0, 10.0, 64),
    ("logistic", (0.8,), [0.015], 0.0, 8.0, 333),
    ("logistic", (1.2,), [0.01], 0.0, 10.0, 17),
]
BATCH_D2 = [
    ("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], 0.0, 7.0, 150),
    ("vanderpol", (1.0,), [2.0, 0.0], 0.0, 6.3, 128),
    ("fitzhughnagumo", (0.7, 0.8, 0.08, 0.5), [1.0, 1.0], 0.0, 20.0, 90),
    ("lotkavolterra", (1.3, 0.9, 2.8, 1.1), [1.2, 0.8], 0.0, 5.0, 61),
    ("vanderpol", (1.2,), [1.9, 0.1], 0.0, 5.0, 257),
    ("fhn_classic", (0.2, 0.2, 3.0), [-1.0, 1.0], 0.0, 5.0, 120),
]


def problems(spec):
    return [(nm, p, y0, np.linspace(t0, t1, N)) for (nm, p, y0, t0, t1, N) in spec]


def close3(x, ref, alts):
    """|x - ref| within 1e-10 relative or 10x the largest spread between ref
    and other reference-faithful orders of the same arithmetic."""
    spread = max(abs(ref - a) for a in alts)
    return abs(float(x) - ref) <= max(TOL * abs(ref), 10.0 * spread, 1e-300)


@pytest.mark.parametrize("spec,q", [(BATCH_D1, 3), (BATCH_D2, 3), (BATCH_D2, 2), (BATCH_D1, 4)])
def test_batch_matches_oracle(spec, q):
    """Every problem of a mixed batch against the oracle: the same IEKS
    iteration count; means, covariances per unit sigma^2, sigma^2 (d = 1),
    NLL and objective within 1e-10 or 10x the spread between three
    bracketings of the reference's arithmetic in the oracle -- its
    associative-scan tree, the sequential scan, and the batched solve's own
    segmented schedule (oracle.blocked.segmented_filtsmooth)."""
    C0, Cg = 4, 2
    res = pbatch.solve_batch(problems(spec), order=q, maxiters=1000, C0=C0, Cg=Cg)
    for b, (nm, p, y0, t0, t1, N) in enumerate(spec):
        o = oracle_ivp(nm, p, y0, t0, t1)
        ts = np.linspace(t0, t1, N)
        (om, oL), oinfo = osolver.solve(o, ts, q, init="constant", maxiters=1000)
        alts = [osolver.solve(o, ts, q, init="constant", maxiters=1000, scan=sequential_scan),
                osolver.solve(o, ts, q, init="constant", maxiters=1000,
                              filtsmooth_fn=oblocked.segmented_filtsmooth(C0, Cg))]
        (gm, gL), ginfo = res.problem(b)
        gm, gL = gm.cpu().numpy(), gL.cpu().numpy()
        assert int(ginfo["iterations"]) == oinfo["iterations"], (b, nm)
        assert rel(gm, om) <= max(TOL, 10 * max(rel(am, om) for (am, _), _ in alts)), (b, nm)
        gs, os_ = float(ginfo["sigma_squared"]), oinfo["sigma_squared"]
        cspread = max(covrel(aL / ai["sigma_squared"], oL / os_) for (_, aL), ai in alts)
        assert covrel(gL / gs, oL / os_) <= max(TOL, 10 * cspread), (b, nm)
        if len(y0) == 1:
            assert close3(gs, os_, [ai["sigma_squared"] for _, ai in alts]), (b, nm)
        assert close3(ginfo["obj"], oinfo["obj"], [ai["obj"] for _, ai in alts]), (b, nm)
        assert close3(ginfo["nll"], oinfo["nll"], [ai["nll"] for _, ai in alts]), (b, nm)


def _run(spec, q, C0=8, Cg=2):
    return pbatch.solve_batch(problems(spec), order=q, maxiters=1000, C0=C0, Cg=Cg)


def _same(ra, a, rb, b):
    (ma, La), ia = ra.problem(a)
    (mb, Lb), ib = rb.problem(b)
    assert torch.equal(ma, mb) and torch.equal(La, Lb)
    for k in ("iterations", "nll", "obj", "sigma_squared"):
        assert float(ia[k]) == float(ib[k]), k


def test_batch_result_independent_of_the_mix():
    """Bit-identical results for a problem solved alone, in the batch, and in
    the batch in reverse order (fixed C0, Cg)."""
    full = _run(BATCH_D2, 3)
    rev = _run(BATCH_D2[::-1], 3)
    B = len(BATCH_D2)
    for b in range(B):
        alone = _run([BATCH_D2[b]], 3)
        _same(full, b, alone, 0)
        _same(full, b, rev, B - 1 - b)


def test_batch_graph_and_direct_launches_agree():
    a = _run(BATCH_D1, 3)
    os.environ["POF_BATCH_NO_GRAPH"] = "1"
    try:
        b = _run(BATCH_D1, 3)
    finally:
        del os.environ["POF_BATCH_NO_GRAPH"]
    for i in range(len(BATCH_D1)):
        _same(a, i, b, i)


def test_batch_matches_plain_solve():
    """Each problem against pof.solver.solve (one IVP per call): same
    iteration count, means within the oracle-spread tolerance."""
    spec = BATCH_D1
    res = pbatch.solve_batch(problems(spec), order=3, maxiters=1000)
    for b, (nm, p, y0, t0, t1, N) in enumerate(spec):
        ivp = pivp.logistic(t0=t0, tmax=t1, y0=y0, r=p[0])
        ts = np.linspace(t0, t1, N)
        out, info = psolver.solve(f=ivp.f, y0=ivp.y0, ts=ts, order=3, init="constant", maxiters=1000)
        (gm, _), ginfo = res.problem(b)
        o = oracle_ivp(nm, p, y0, t0, t1)
        (om, _), _ = osolver.solve(o, ts, 3, init="constant", maxiters=1000)
        (sm, _), _ = osolver.solve(o, ts, 3, init="constant", maxiters=1000, scan=sequential_scan)
        assert int(ginfo["iterations"]) == int(info["iterations"])
        assert rel(gm.cpu().numpy(), out.mean.cpu().numpy()) <= max(TOL, 20 * rel(sm, om))


def test_batch_chunk_shapes():
    """Chunk lengths 1, 3, 64 and group sizes 2, 5 (ragged problems whose
    step counts are not multiples of either) agree to 1e-10 (well-conditioned
    problems: the oracle's own orders agree to ~1e-14)."""
    spec = BATCH_D1
    ref = None
    for C0, Cg in [(1, 2), (3, 5), (64, 2), (3, 2)]:
        res = _run(spec, 3, C0=C0, Cg=Cg)
        if ref is None:
            ref = res
            continue
        for b in range(len(spec)):
            (ma, _), ia = ref.problem(b)
            (mb, _), ib = res.problem(b)
            assert int(ia["iterations"]) == int(ib["iterations"])
            assert rel(mb.cpu().numpy(), ma.cpu().numpy()) <= TOL


# well-resolved problems (the float64 fixed point is the ODE solution): the
# float32 phase must not move the IEKS to another fixed point
MIXED_D2 = [
    ("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], 0.0, 7.0, 600),
    ("vanderpol", (1.0,), [2.0, 0.0], 0.0, 6.3, 128),
    ("fitzhughnagumo", (0.7, 0.8, 0.08, 0.5), [1.0, 1.0], 0.0, 20.0, 90),
    ("lotkavolterra", (1.3, 0.9, 2.8, 1.1), [1.2, 0.8], 0.0, 5.0, 300),
    ("vanderpol", (1.2,), [1.9, 0.1], 0.0, 5.0, 257),
    ("fhn_classic", (0.2, 0.2, 3.0), [-1.0, 1.0], 0.0, 5.0, 120),
]


@pytest.mark.parametrize("spec,q", [(MIXED_D2, 3), (BATCH_D1, 3)])
def test_batch_mixed_precision(spec, q):
    """Float32 iterations + float64 polish per problem: within 1e-6 (max
    relative error of the solution y) of the float64 batch, which is the
    oracle's fixed point (test_batch_matches_oracle)."""
    ref = pbatch.solve_batch(problems(spec), order=q, maxiters=1000)
    mix = pbatch.solve_batch(problems(spec), order=q, maxiters=1000, precision="mixed")
    it32 = mix.info["iterations_float32"].cpu().numpy()
    assert (it32 >= 0).all()
    errs = []
    for b in range(len(spec)):
        (ma, _), _ = ref.problem(b)
        (mb, _), _ = mix.problem(b)
        errs.append((rel(mb.cpu().numpy(), ma.cpu().numpy()), spec[b][0], int(it32[b]),
                     int(mix.info["iterations"][b]), int(ref.info["iterations"][b])))
    print(errs)
    assert all(e[0] <= 1e-6 for e in errs), errs
    # the float32 phase does the bulk of the work on these problems
    assert it32.sum() > 0


def test_batch_mixed_settled_float32_phase():
    """settle_f32 = 0.1 (non-shrinking float32 changes counted only below a
    10 % change): more float32 iterations, and on these well-resolved
    problems still the float64 fixed point to 1e-6."""
    spec, q = MIXED_D2, 3
    ref = pbatch.solve_batch(problems(spec), order=q, maxiters=1000)
    mix = pbatch.solve_batch(problems(spec), order=q, maxiters=1000, precision="mixed", settle_f32=0.1)
    base = pbatch.solve_batch(problems(spec), order=q, maxiters=1000, precision="mixed")
    assert int(mix.info["iterations_float32"].sum()) >= int(base.info["iterations_float32"].sum())
    for b in range(len(spec)):
        (ma, _), _ = ref.problem(b)
        (mb, _), _ = mix.problem(b)
        assert rel(mb.cpu().numpy(), ma.cpu().numpy()) <= 1e-6, (b, spec[b][0])


def test_batch_mixed_independent_of_the_mix():
    full = pbatch.solve_batch(problems(MIXED_D2), order=3, maxiters=1000, C0=8, precision="mixed")
    for b in (0, 3):
        alone = pbatch.solve_batch(problems([MIXED_D2[b]]), order=3, maxiters=1000, C0=8, precision="mixed")
        _same(full, b, alone, 0)
        assert int(full.info["iterations_float32"][b]) == int(alone.info["iterations_float32"][0])


def test_autotune_picks_a_candidate_and_keeps_parity(tmp_path, monkeypatch):
    """Chunk length, group size and level-0 team width by timing; the tuned
    solve keeps parity; solve_batch(C0="auto") stores the choice in the
    autotune cache and takes it from there the next time."""
    prep = pbatch.prepare_batch(problems(BATCH_D2), 3)
    C0, Cg, wide, times = pbatch.autotune(prep, C0s=(4, 16), Cgs=(2, 4), iterations=2, repeats=1)
    assert (C0, Cg, wide) in times and len(times) == 8 and all(t > 0 for t in times.values())
    with pbatch._TeamWidth(wide):
        res = pbatch.solve_batch(problems(BATCH_D2), order=3, maxiters=1000, C0=C0, Cg=Cg)
    monkeypatch.setenv("POF_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    auto = pbatch.solve_batch(problems(BATCH_D2), order=3, maxiters=1000, C0="auto")
    assert pbatch.load_tuning(prep) is not None
    again = pbatch.solve_batch(problems(BATCH_D2), order=3, maxiters=1000, C0="auto")
    assert torch.equal(auto.mean, again.mean)  # the cached choice, the same bits
    ref = pbatch.solve_batch(problems(BATCH_D2), order=3, maxiters=1000, C0=4, Cg=2)
    for b in range(len(BATCH_D2)):
        (ma, _), ia = ref.problem(b)
        (mb, _), ib = res.problem(b)
        assert int(ia["iterations"]) == int(ib["iterations"])
        assert rel(mb.cpu().numpy(), ma.cpu().numpy()) <= TOL
