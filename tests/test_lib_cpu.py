"""libpof.so loads and exports every entry point of include/pof.h; host-side
logic that needs no GPU (CPU only)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pof.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(pof_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from pof import _build, _lib

    _build.build(verbose=False)  # no-op when up to date
    return _lib.lib()


def test_header_declares_entry_points():
    names = header_functions()
    for n in ("pof_linear_filtsmooth", "pof_linear_noiseless_filtering", "pof_smoothing", "pof_ieks_solve",
              "pof_linearize", "pof_sequential_linear_filtsmooth", "pof_sequential_eks"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from pof import _lib

    assert set(header_functions()) == set(_lib.exported_symbols())


def test_status_strings(lib):
    assert lib.pof_status_string(0) == b"ok"
    assert b"workspace" in lib.pof_status_string(-3)
    assert lib.pof_version() >= 1


def test_shapes_and_workspace_queries(lib):
    from pof import _lib

    assert _lib.shape_supported(8, 2) and _lib.shape_supported(4, 1)
    assert not _lib.shape_supported(7, 2)
    w1 = lib.pof_filtsmooth_workspace_bytes(0, 999, 8, 2)
    w2 = lib.pof_filtsmooth_workspace_bytes(0, 9999, 8, 2)
    assert 0 < w1 < w2
    assert lib.pof_ieks_workspace_bytes(0, 999, 8, 2) > w1
    assert lib.pof_filtsmooth_workspace_bytes(0, 0, 8, 2) == 0


def test_parallel_top_option_changes_the_plan(lib, monkeypatch):
    """POF_KS (read at each call): 0, the default, keeps the binary tree to two
    top elements; -1 stops it at the first level of at most 16384 / team lanes
    elements and adds the parallel scan's ping-pong buffer, which at N = 2^16,
    D = 8 costs less than the dropped levels' buffers."""
    dflt = lib.pof_filtsmooth_workspace_bytes(0, 65535, 8, 2)
    monkeypatch.setenv("POF_KS", "0")
    assert lib.pof_filtsmooth_workspace_bytes(0, 65535, 8, 2) == dflt
    monkeypatch.setenv("POF_KS", "-1")
    ks = lib.pof_filtsmooth_workspace_bytes(0, 65535, 8, 2)
    assert ks != dflt and ks > 0
    monkeypatch.setenv("POF_KS", "2")  # not above the two-element top: the tree
    assert lib.pof_filtsmooth_workspace_bytes(0, 65535, 8, 2) == dflt


def test_flop_model_counts_skipped_zeros_out():
    """The flop model counts the team kernels' operations without the
    structural zeros they skip: fewer than the dense loops from D = 6 on,
    equal below (thread-per-chunk level 0 runs the dense loops)."""
    from pof import _flops

    for D, d in ((8, 2), (6, 2), (10, 2)):
        assert _flops.kf_step(D, d, True) < _flops.kf_step(D, d, True, structured=False)
        assert _flops.cond_fold_step(D, d) < _flops.cond_fold_step(D, d, structured=False)
    assert _flops.kf_step(4, 1, True) == _flops.kf_step(4, 1, True, structured=False)
    # a lower-triangular right block: reflector j spans columns j+1 .. D+j
    assert _flops.tria(8, 16, wlow=8) < _flops.tria(8, 16)
    assert _flops.tria(8, 16, wlow=15) == _flops.tria(8, 16)
    # zero columns from ncut on: the reflectors from ncut - 1 on vanish
    assert _flops.tria(10, 10, ncut=8) == _flops.tria(7, 10, MB=3, ncut=8)


def test_argument_errors_without_gpu(lib):
    """Invalid arguments are rejected on the host before any CUDA call."""
    null = ctypes.c_void_p(0)
    rc = lib.pof_linear_filtsmooth(0, 10, 7, 2, null, null, null, null, 0, null, null, null, 0, null, null, null,
                                   null, 0, null)
    assert rc == -2  # shape not compiled
    rc = lib.pof_linear_filtsmooth(5, 10, 8, 2, null, null, null, null, 0, null, null, null, 0, null, null, null,
                                   null, 0, null)
    assert rc == -6  # dtype
    rc = lib.pof_linear_filtsmooth(0, 10, 8, 2, null, null, null, null, 0, null, null, null, 0, null, null, null,
                                   null, 0, null)
    assert rc == -1  # null pointers
    rc = lib.pof_linearize(0, 10, 8, 2, 1, null, 0.1, null, null, null, null)
    assert rc == -5  # logistic is d = 1


def test_transitions_match_oracle():
    import numpy as np
    import torch

    from oracle import core
    from pof import transitions as tr

    iwp = tr.IWP(wiener_process_dimension=2, num_derivatives=3)
    A, L = tr.preconditioned_discretize(iwp, device=torch.device("cpu"))
    oA, oL = core.preconditioned_discretize(2, 3)
    assert np.array_equal(A.numpy(), oA) and np.array_equal(L.numpy(), oL)
    P, PI = tr.nordsieck_preconditioner(iwp, 0.1, device=torch.device("cpu"))
    oP, oPI = core.nordsieck_preconditioner(2, 3, 0.1)
    assert np.allclose(P.numpy(), oP, rtol=1e-15) and np.allclose(PI.numpy(), oPI, rtol=1e-15)


@pytest.mark.parametrize("name,ctor,q", [("fhn_classic", "fhn_classic", 4), ("logistic", "logistic", 3),
                                         ("threebody", "threebody", 3), ("lotkavolterra", "lotkavolterra", 5)])
def test_taylor_mode_matches_oracle(name, ctor, q):
    """torch.func nested-jvp Taylor mode == the oracle's Taylor arithmetic."""
    import numpy as np

    from oracle import ivp as oivp, taylor
    from pof import initialization, ivp

    p = getattr(ivp, ctor)()
    o = getattr(oivp, ctor)()
    a = initialization.taylor_derivatives(p.f, p.y0, q).numpy()
    b = taylor.taylor_derivatives(o.components, o.y0, q)
    assert np.allclose(a, b, rtol=1e-13, atol=1e-13)


def test_sizes_strides_and_workspace_checked_before_any_cuda_call(lib):
    """Empty inputs (n_steps = 0), strides that are neither 0 nor one
    matrix, a workspace below the query's size, a negative maxiters and a
    field of the wrong dimension are refused on the host with their status,
    before any pointer is used (the pointers here are placeholders)."""
    import ctypes as C

    from pof import _lib

    ARG, WORKSPACE, FIELD, DTYPE = -1, -3, -5, -6  # POF_ERR_* of include/pof.h
    P = 256  # never dereferenced: every call below returns before any CUDA call
    dp = C.cast(C.c_void_p(P), C.POINTER(C.c_double))
    n, D, d = 100, 8, 2
    ws = lib.pof_filtsmooth_workspace_bytes(0, n, D, d)

    def fs(n=n, fts=0, rs=0, wsb=ws, R=P):
        return lib.pof_linear_filtsmooth(0, n, D, d, P, P, P, P, fts, P, P, R, rs, P, P, dp, P, wsb, None)

    assert fs(n=0) == ARG
    assert fs(n=-5) == ARG
    assert fs(fts=D) == ARG
    assert fs(rs=d) == ARG
    assert fs(wsb=ws - 1) == WORKSPACE
    assert lib.pof_linear_noiseless_filtering(0, n, D, d, P, P, P, P, 0, P, P, None, 0, P, P, dp, P, ws - 1,
                                              None) == WORKSPACE
    sws = lib.pof_filtsmooth_workspace_bytes(0, n, D, 1)
    assert lib.pof_smoothing(0, 0, D, P, P, 0, P, P, P, P, dp, P, sws, None) == ARG
    assert lib.pof_smoothing(0, n, D, P, P, 7, P, P, P, P, dp, P, sws, None) == ARG

    iws = lib.pof_ieks_workspace_bytes(0, n, D, d)
    fhn = _lib.FIELDS["fhn_classic"]

    def solve(n=n, field=fhn, maxiters=10, wsb=iws, dtype=0):
        return lib.pof_ieks_solve(dtype, n, D, d, field, P, 0.1, P, P, P, P, P, P, maxiters, 1, dp, P, wsb, None)

    assert solve(n=0) == ARG
    assert solve(maxiters=-1) == ARG
    assert solve(wsb=iws - 1) == WORKSPACE
    assert solve(field=_lib.FIELDS["logistic"]) == FIELD
    assert solve(field=999) == FIELD
    assert solve(dtype=3) == DTYPE

    mws = lib.pof_ieks_mixed_workspace_bytes(n, D, d)

    def mixed(rtol=1e-5, settle=1.0, wsb=mws):
        return lib.pof_ieks_solve_mixed(n, D, d, fhn, P, 0.1, P, P, P, P, P, P, 10, rtol, settle, 10, 1, dp, P, wsb,
                                        None)

    assert mixed(rtol=0.0) == ARG
    assert mixed(settle=float("nan")) == ARG
    assert mixed(wsb=mws - 1) == WORKSPACE


REFERENCE_API = {
    # the reference's public names per module (pof/*.py), as this package provides them
    "pof.solver": ["solve", "sequential_eks_solve"],
    "pof.parallel_filtsmooth": ["linear_filtsmooth", "linear_noiseless_filtering", "smoothing"],
    "pof.parallel_filtsmooth.filter": ["linear_noiseless_filtering", "sqrt_filtering_operator"],
    "pof.parallel_filtsmooth.smoother": ["smoothing", "get_elements", "sqrt_smoothing_operator"],
    "pof.sequential_filtsmooth": ["filtsmooth", "linear_filtsmooth"],
    "pof.sequential_filtsmooth.filter": ["extended_kalman_filter", "linear_noiseless_filter"],
    "pof.sequential_filtsmooth.smoother": ["smoothing"],
    "pof.step": ["linearize_at_previous_states", "inflate", "ieks_step"],
    "pof.iterators": ["fs", "lom", "lom_reg", "ieks_iterator", "qpm_ieks_iterator", "lm_ieks_iterator"],
    "pof.observations": ["NonlinearModel", "AffineModel", "linearize", "uncertain_linearize", "linearize_ek0",
                         "linearize_regularized"],
    "pof.transitions": ["TransitionModel", "IWP", "hilbert", "pascal", "preconditioned_discretize_1d",
                        "preconditioned_discretize", "nordsieck_preconditioner_1d", "nordsieck_preconditioner",
                        "non_preconditioned_discretize", "projection_matrix_1d", "projection_matrix",
                        "get_transition_model", "discretize_transitions"],
    "pof.convergence_criteria": ["crit"],
    "pof.convenience": ["linearize_observation_model", "set_up_solver", "set_up_solver_no_precond",
                        "get_initial_trajectory"],
    "pof.initialization": ["taylor_mode_init", "uncertain_init", "constant_init", "classic_to_init", "prior_init",
                           "updated_prior_init", "coarse_ekf_init"],
    "pof.ivp": ["logistic", "lotkavolterra", "vanderpol", "fitzhughnagumo", "rober", "rigid_body", "seir",
                "threebody", "henonheiles"],
    "pof.utils": ["MVNSqrt", "AffineModel", "mvn_loglikelihood", "tria", "qr", "linearize",
                  "append_zeros_along_new_axis", "objective_function_value", "_gmul", "whiten",
                  "cholesky_update_many"],
}


@pytest.mark.parametrize("module", sorted(REFERENCE_API))
def test_reference_api_names_exist(module):
    import importlib

    mod = importlib.import_module(module)
    missing = [n for n in REFERENCE_API[module] if not hasattr(mod, n)]
    assert not missing, missing


def test_dense_entry_argument_errors_without_gpu(lib):
    """The dense path's entry points check their arguments and workspace on
    the host before any CUDA call; uncompiled shapes with D >= 32 reach it
    through pof_linear_filtsmooth (a null pointer is then POF_ERR_ARG, not
    POF_ERR_SHAPE)."""
    null = ctypes.c_void_p(0)
    one = ctypes.c_void_p(256)  # never dereferenced: every call below fails its checks first
    assert lib.pof_shape_supported(48, 6) == 0
    rc = lib.pof_linear_filtsmooth(0, 10, 48, 6, null, null, null, null, 0, null, null, null, 0, null, null, null,
                                   null, 0, null)
    assert rc == -1
    rc = lib.pof_linear_filtsmooth(0, 10, 31, 6, null, null, null, null, 0, null, null, null, 0, null, null, null,
                                   null, 0, null)
    assert rc == -2  # below the dense path's D
    args = [0, 10, 48, 6] + [one] * 4 + [0] + [one] * 3 + [0] + [one] * 3
    assert lib.pof_dense_linear_filtsmooth(3, *args, 0, one, 1 << 40, null) == -1     # which
    assert lib.pof_dense_linear_filtsmooth(1, 7, *args[1:], 0, one, 1 << 40, null) == -6  # dtype
    assert lib.pof_dense_linear_filtsmooth(1, *args, -1, one, 1 << 40, null) == -1    # chunks
    bad = list(args)
    bad[8] = 7  # ft_stride neither 0 nor D * D
    assert lib.pof_dense_linear_filtsmooth(1, *bad, 0, one, 1 << 40, null) == -1
    need = lib.pof_dense_workspace_bytes(0, 1, 10, 48, 6, 0)
    assert need > 0 and lib.pof_filtsmooth_workspace_bytes(0, 10, 48, 6) == need
    assert lib.pof_dense_linear_filtsmooth(1, *args, 0, one, need - 1, null) == -3   # workspace
    assert lib.pof_dense_workspace_bytes(0, 5, 10, 48, 6, 0) == 0
    # more chunks, more per-chunk buffers; float32 half the bytes per element
    assert lib.pof_dense_workspace_bytes(0, 1, 4096, 64, 8, 256) > lib.pof_dense_workspace_bytes(0, 1, 4096, 64, 8, 16)
    assert lib.pof_dense_workspace_bytes(1, 1, 4096, 64, 8, 64) < lib.pof_dense_workspace_bytes(0, 1, 4096, 64, 8, 64)
    rc = lib.pof_linearize(0, 10, 40, 7, 11, one, 0.1, one, one, one, null)
    assert rc == -5  # the reaction-diffusion field needs an even d
