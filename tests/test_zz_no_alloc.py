"""The allocation-free filter/smoother entry point (collected last).

pof_linear_filtsmooth_noalloc serves callers that cannot allocate device
memory (plugin hosts that pass only inputs and outputs, a foreign
allocator, real-time loops that must not call cudaMalloc):
its scratch is a fixed array inside libpof.  Called twice in a row through
the C ABI, it must give the results of pof_linear_filtsmooth, which uses a
caller-provided workspace, and it must refuse problems larger than its
scratch."""

import ctypes

import numpy as np
import pytest
import torch

from oracle import ivp as oivp, solver as osolver
from pof import _lib

pytestmark = pytest.mark.gpu


def _inputs(ivp, N, q):
    ts = np.linspace(ivp.t0, ivp.tmax, N)
    st = osolver.set_up_solver(ivp, ts, q)
    states = osolver.get_initial_trajectory(st, "constant")
    for _ in range(3):
        states, _, _, _ = osolver.ieks_step(st, states)
    H, c, R = osolver.linearize_at_previous_states(st, states[0])
    dev = torch.device("cuda", 0)
    T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)  # noqa: E731
    return dict(x0m=T(st.x0[0]), x0L=T(st.x0[1]), F=T(st.F[0]), QL=T(st.QL[0]), H=T(H), c=T(c), R=T(R))


def _run(lib, a, n, D, d, noalloc):
    means = torch.empty((n + 1, D), dtype=torch.float64, device="cuda")
    chols = torch.empty((n + 1, D, D), dtype=torch.float64, device="cuda")
    scal = torch.zeros(_lib.S_COUNT, dtype=torch.float64, device="cuda")
    p = _lib.ptr
    common = (0, n, D, d, p(a["x0m"]), p(a["x0L"]), p(a["F"]), p(a["QL"]), 0, p(a["H"]), p(a["c"]), p(a["R"]),
              d * d, p(means), p(chols), p(scal))
    if noalloc:
        rc = lib.pof_linear_filtsmooth_noalloc(*common, _lib.stream_handle())
    else:
        wsb = lib.pof_filtsmooth_workspace_bytes(0, n, D, d)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        rc = lib.pof_linear_filtsmooth(*common, p(ws), wsb, _lib.stream_handle())
    torch.cuda.synchronize()
    return rc, means.cpu().numpy(), chols.cpu().numpy(), scal.cpu().numpy()


@pytest.mark.parametrize("name,mk,N,q", [("fhn", lambda: oivp.fhn_classic(tmax=10.0), 501, 3),
                                         ("logistic", lambda: oivp.logistic(r=3.0), 2000, 2)])
def test_noalloc_matches_workspace_entry_point_twice(name, mk, N, q):
    torch.cuda.set_device(0)
    lib = _lib.lib()
    ivp = mk()
    a = _inputs(ivp, N, q)
    n, d, D = N - 1, ivp.y0.shape[0], ivp.y0.shape[0] * (q + 1)
    rc, m_ref, L_ref, s_ref = _run(lib, a, n, D, d, noalloc=False)
    assert rc == 0
    for _ in range(2):  # the shared scratch keeps the previous call's contents
        rc, m, L, s = _run(lib, a, n, D, d, noalloc=True)
        assert rc == 0, lib.pof_status_string(rc)
        assert np.abs(m - m_ref).max() <= 1e-10 * np.abs(m_ref).max()
        assert np.abs(L @ np.swapaxes(L, -1, -2) - L_ref @ np.swapaxes(L_ref, -1, -2)).max() <= \
            1e-10 * np.abs(L_ref @ np.swapaxes(L_ref, -1, -2)).max()
        assert np.allclose(s[:4], s_ref[:4], rtol=1e-10, atol=0)


SCRATCH = 16 * 1024 * 1024


def _n_max(lib, dtype, D, d):
    """Largest step count whose workspace fits the fixed scratch."""
    lo, hi = 1, 10**8
    while lo < hi:
        m = (lo + hi + 1) // 2
        if lib.pof_filtsmooth_workspace_bytes(dtype, m, D, d) <= SCRATCH:
            lo = m
        else:
            hi = m - 1
    return lo


def test_noalloc_refuses_problems_larger_than_its_scratch():
    lib = _lib.lib()
    null = ctypes.c_void_p(0)

    def call(dtype, n, D, d):
        return lib.pof_linear_filtsmooth_noalloc(dtype, n, D, d, null, null, null, null, 0, null, null, null, 0,
                                                 null, null, null, null)

    for dtype, D, d, documented in ((0, 8, 2, 3344), (1, 8, 2, 6660), (0, 4, 1, 20296), (0, 3, 1, 34212)):
        n_max = _n_max(lib, dtype, D, d)
        assert n_max == documented  # the limits include/pof.h lists
        assert call(dtype, n_max + 1, D, d) == -3  # POF_ERR_WORKSPACE, refused before any GPU work
    assert call(0, 10_000_000, 8, 2) == -3
    # bad inputs get the statuses of the workspace entry point, not the size refusal
    for args in ((7, 100, 8, 2), (0, 0, 8, 2), (0, 100, 8, 9), (0, 100, 7, 2)):
        dtype, n, D, d = args
        ref = lib.pof_linear_filtsmooth(dtype, n, D, d, null, null, null, null, 0, null, null, null, 0, null, null,
                                        null, null, 0, null)
        assert call(*args) == ref != 0, (args, ref)


def test_noalloc_runs_the_largest_problem_it_accepts():
    """The boundary itself: n_max steps (D = 8, d = 2, float64) run in the
    fixed scratch and equal the workspace entry point."""
    torch.cuda.set_device(0)
    lib = _lib.lib()
    n = _n_max(lib, 0, 8, 2)
    a = _inputs(oivp.fhn_classic(tmax=10.0 * n / 500), n + 1, 3)
    rc, m_ref, L_ref, s_ref = _run(lib, a, n, 8, 2, noalloc=False)
    assert rc == 0
    rc, m, L, s = _run(lib, a, n, 8, 2, noalloc=True)
    assert rc == 0, lib.pof_status_string(rc)
    assert np.abs(m - m_ref).max() <= 1e-10 * np.abs(m_ref).max()
    assert np.allclose(s[:4], s_ref[:4], rtol=1e-10, atol=0)
