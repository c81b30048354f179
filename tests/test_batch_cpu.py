"""Host side of the batched solve (CPU only): the batch set-up against the
oracle's one-problem set-up, the workspace query and the argument checks of
pof_ieks_solve_batch (which return before any GPU work)."""

import ctypes

import numpy as np
import torch
import pytest

from oracle import ivp as oivp, solver as osolver


@pytest.fixture(scope="module")
def lib():
    from pof import _build, _lib

    _build.build(verbose=False)
    return _lib.lib()


PROBLEMS = [
    ("fhn_classic", (0.2, 0.2, 3.0), [-1.0, 1.0], np.linspace(0.0, 100.0, 300)),
    ("fhn_classic", (0.17, 0.23, 2.7), [-0.9, 1.1], np.linspace(0.0, 100.0, 1001)),
    ("lotkavolterra", (1.5, 1.0, 3.0, 1.0), [1.0, 1.0], np.linspace(0.0, 7.0, 33)),
    ("vanderpol", (10.0,), [2.0, 0.0], np.linspace(0.0, 6.3, 64)),
]


def oracle_of(name, p, y0, ts):
    if name == "fhn_classic":
        return oivp.fhn_classic(tmax=ts[-1], y0=y0, a=p[0], b=p[1], c=p[2])
    if name == "lotkavolterra":
        return oivp.lotkavolterra(tmax=ts[-1], y0=y0, p=p)
    if name == "vanderpol":
        return oivp.vanderpol(tmax=ts[-1], y0=y0, stiffness_constant=p[0])
    raise ValueError(name)


@pytest.mark.parametrize("q", [2, 3, 4])
def test_prepare_batch_matches_oracle_setup(q):
    """x0 (Taylor mode, times P^-1), the constant-init trajectories, F, QL and
    the projection scale p0 of every problem equal the oracle's set-up."""
    import torch

    from pof import batch as pbatch

    prep = pbatch.prepare_batch(PROBLEMS, q, device=torch.device("cpu"))
    assert prep["D"] == 2 * (q + 1)
    off = prep["offsets"]
    for b, (nm, p, y0, ts) in enumerate(PROBLEMS):
        st = osolver.set_up_solver(oracle_of(nm, p, y0, ts), ts, q)
        np.testing.assert_allclose(prep["x0m"][b].numpy(), st.x0[0], rtol=1e-13, atol=0)
        m0, _ = osolver.get_initial_trajectory(st, "constant")
        np.testing.assert_allclose(prep["means0"][off[b]:off[b + 1]].numpy(), m0, rtol=1e-14, atol=0)
        np.testing.assert_array_equal(prep["F"].numpy(), st.F[0])
        np.testing.assert_array_equal(prep["QL"].numpy(), st.QL[0])
        assert float(prep["p0"][b]) == pytest.approx(st.P[0, 0], rel=1e-15)
        assert prep["n_steps"][b] == len(ts) - 1


def _arr(a, t):
    a = np.ascontiguousarray(a, dtype=t)
    return a, a.ctypes.data_as(ctypes.c_void_p)


def test_batch_workspace_query(lib):
    ns, pns = _arr([299, 1000, 32, 63], np.int64)
    w = lib.pof_batch_workspace_bytes(0, 4, pns, 8, 2, 0, 0)
    w_small = lib.pof_batch_workspace_bytes(0, 2, pns, 8, 2, 0, 0)
    assert 0 < w_small < w
    assert lib.pof_batch_workspace_bytes(1, 4, pns, 8, 2, 0, 0) < w  # float32
    assert lib.pof_batch_workspace_bytes(0, 4, pns, 7, 2, 0, 0) == 0  # shape not compiled
    bad, pbad = _arr([299, 0], np.int64)
    assert lib.pof_batch_workspace_bytes(0, 2, pbad, 8, 2, 0, 0) == 0  # empty problem
    assert lib.pof_batch_workspace_bytes(0, 0, pns, 8, 2, 0, 0) == 0


def test_batch_argument_errors_without_gpu(lib):
    """Every refusal happens on the host before any CUDA call."""
    ns, pns = _arr([10, 20], np.int64)
    fl, pfl = _arr([5, 5], np.int32)
    hh, ph = _arr([0.1, 0.05], np.float64)
    fake = ctypes.c_void_p(256)  # never dereferenced: the calls fail first

    def call(dtype=0, B=2, n=pns, D=8, d=2, fields=pfl, params=fake, h=ph, ws=fake, wsb=1 << 30):
        return lib.pof_ieks_solve_batch(dtype, B, n, D, d, fields, params, h, fake, fake, fake, fake, fake, fake,
                                        100, 1, 0, 0, None, ws, wsb, None)

    assert call(dtype=3) == -6
    assert call(D=7) == -1 and call(D=12, d=2) == -2
    assert call(params=None) == -1
    bf, pbf = _arr([5, 1], np.int32)  # logistic has d = 1
    assert call(fields=pbf) == -5
    assert call(wsb=16) == -3
    z, pz = _arr([0.1, 0.0], np.float64)
    assert call(h=pz) == -1
    neg, pneg = _arr([10, -1], np.int64)
    assert call(n=pneg) == -1


def test_projection_and_per_problem_results():
    """project() applies each problem's E0 P to its rows (as pof.solver.solve
    returns gmul_stack(E0 P, states)) and BatchResult.problem(b) slices
    problem b's rows and info out of the concatenation."""
    import torch

    from pof import batch as pbatch

    q = 3
    prep = pbatch.prepare_batch(PROBLEMS, q, device=torch.device("cpu"))
    G, D = prep["means0"].shape
    g = torch.Generator().manual_seed(5)
    means = torch.randn((G, D), dtype=torch.float64, generator=g)
    chols = torch.randn((G, D, D), dtype=torch.float64, generator=g)
    ym, yc = pbatch.project(prep, means, chols)
    info = {"iterations": torch.arange(len(PROBLEMS)), "nll": torch.zeros(len(PROBLEMS)), "calibrated": True}
    res = pbatch.BatchResult(ym, yc, prep["offsets"], info)
    off = prep["offsets"]
    for b, (nm, p, y0, ts) in enumerate(PROBLEMS):
        E0 = osolver.set_up_solver(oracle_of(nm, p, y0, ts), ts, q).E0
        s, e = off[b], off[b + 1]
        (mb, cb), ib = res.problem(b)
        np.testing.assert_allclose(mb.numpy(), means[s:e].numpy() @ E0.T, rtol=1e-14, atol=1e-300)
        np.testing.assert_allclose(cb.numpy(), E0 @ chols[s:e].numpy(), rtol=1e-14, atol=1e-300)
        assert int(ib["iterations"]) == b and ib["calibrated"] is True


def test_server_and_mixed_workspace_queries_and_refusals(lib):
    """The serving engine's and the mixed-precision batch's size queries, and
    pof_server_create's refusals, which all happen on the host before any
    CUDA call (placeholder pointers are never used)."""
    w = lib.pof_server_workspace_bytes(8, 2, 16, 100_000, 1 << 20)
    assert w > 0
    assert lib.pof_server_workspace_bytes(8, 2, 32, 100_000, 1 << 20) > w
    assert lib.pof_server_workspace_bytes(8, 2, 16, 200_000, 1 << 20) > w
    assert lib.pof_server_workspace_bytes(8, 2, 16, 100_000, 1 << 24) > w
    assert lib.pof_server_workspace_bytes(7, 2, 16, 100_000, 1 << 20) == 0  # shape not compiled
    assert lib.pof_server_workspace_bytes(8, 2, 0, 100_000, 1 << 20) == 0
    assert lib.pof_server_workspace_bytes(8, 2, 16, 1, 1 << 20) == 0
    P = 256
    h = ctypes.c_void_p()
    assert lib.pof_server_create(8, 2, 16, 100_000, 1 << 20, P, P, 1, P, w, None) == -1  # no out pointer
    assert lib.pof_server_create(7, 2, 16, 100_000, 1 << 20, P, P, 1, P, w, ctypes.byref(h)) == -2
    assert lib.pof_server_create(8, 2, 0, 100_000, 1 << 20, P, P, 1, P, w, ctypes.byref(h)) == -1
    assert lib.pof_server_create(8, 2, 16, 100_000, 1 << 20, P, P, 1, P, w - 1, ctypes.byref(h)) == -3
    assert h.value is None

    ns, pns = _arr([299, 1000, 32, 63], np.int64)
    w64 = lib.pof_batch_workspace_bytes(0, 4, pns, 8, 2, 0, 0)
    wmx = lib.pof_batch_mixed_workspace_bytes(4, pns, 8, 2, 0, 0)
    assert wmx > w64 > 0
    assert lib.pof_batch_mixed_workspace_bytes(4, pns, 7, 2, 0, 0) == 0


def test_autotune_cache_round_trip(tmp_path, monkeypatch):
    """The autotuner's choice is stored under the batch's key (GPU, D, d,
    total steps to a factor of two) and found again; a batch of another key
    is tuned anew; other keys of the file are kept."""
    from pof import batch as pbatch

    monkeypatch.setenv("POF_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    prep = {"D": 8, "d": 2, "n_steps": np.array([1000, 3000]), "x0m": torch.zeros(2, 8)}
    other = {"D": 8, "d": 2, "n_steps": np.array([100000]), "x0m": torch.zeros(1, 8)}
    calls = []

    def timer(C0, Cg, wide):
        calls.append((C0, Cg, wide))
        return abs(C0 - 32) + (0.5 if Cg == 4 else 0.0) + (0.25 if wide else 0.0)

    assert pbatch.load_tuning(prep) is None
    assert pbatch.tuned(prep, timer=timer) == (32, 2, False)
    n = len(calls)
    assert n == 5 * 2 * 2
    assert pbatch.tuned(prep, timer=timer) == (32, 2, False) and len(calls) == n  # from the cache
    assert pbatch.autotune_key(other) != pbatch.autotune_key(prep)
    pbatch.tuned(other, timer=timer)
    assert len(calls) == 2 * n
    assert pbatch.load_tuning(prep) == (32, 2, False) and pbatch.load_tuning(other) is not None
