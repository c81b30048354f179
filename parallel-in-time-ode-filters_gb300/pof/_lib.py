"""ctypes binding of libpof.so (the C ABI declared in include/pof.h).

The library is loaded from this package directory.  There is no CPU fallback:
every entry point raises if the library is missing or a call fails.
"""

import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpof.so")

POF_OK = 0
POF_F64, POF_F32 = 0, 1

# out_scalars layout (POF_S_*)
S_NLL, S_OBJ, S_SSQ, S_FOBJ, S_NOTCLOSE = 0, 1, 2, 3, 4
S_COUNT = 8
# info layout (POF_I_*)
I_ITERATIONS, I_NLL, I_OBJ, I_SSQ, I_STATUS = 0, 1, 2, 3, 4
I_COUNT = 5
# info[I_STATUS]: why a problem's IEKS loop stopped (POF_SOLVE_*)
SOLVE_STATUS = {0: "converged", 1: "maxiters", 2: "nonfinite", 3: "cancelled"}

FIELDS = {
    "user": 0,
    "logistic": 1,
    "lotkavolterra": 2,
    "vanderpol": 3,
    "fitzhughnagumo": 4,
    "fhn_classic": 5,
    "rober": 6,
    "rigid_body": 7,
    "seir": 8,
    "threebody": 9,
    "henonheiles": 10,
    "fhn_rd": 11,
}
# Built-in fields with a state dimension of the caller's choosing: linearized
# by pof_linearize at any shape, solved by the host-driven IEKS loop
# (pof.solver), never by the device loops.
DENSE_FIELDS = frozenset({"fhn_rd"})


class PofError(RuntimeError):
    pass


_lib = None

_c = ctypes
_i32, _i64, _sz, _vp, _dp, _f64 = _c.c_int32, _c.c_int64, _c.c_size_t, _c.c_void_p, _c.c_void_p, _c.c_double

_SIGS = {
    "pof_status_string": (_c.c_char_p, [_c.c_int]),
    "pof_last_cuda_error": (_c.c_char_p, []),
    "pof_version": (_c.c_int, []),
    "pof_shape_supported": (_c.c_int, [_i32, _i32]),
    "pof_filtsmooth_workspace_bytes": (_sz, [_i32, _i64, _i32, _i32]),
    "pof_ieks_workspace_bytes": (_sz, [_i32, _i64, _i32, _i32]),
    "pof_linear_filtsmooth": (
        _c.c_int,
        [_i32, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _dp, _vp, _sz, _vp],
    ),
    "pof_linear_noiseless_filtering": (
        _c.c_int,
        [_i32, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _dp, _vp, _sz, _vp],
    ),
    "pof_linear_filtsmooth_noalloc": (
        _c.c_int,
        [_i32, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _dp, _vp],
    ),
    "pof_smoothing": (_c.c_int, [_i32, _i64, _i32, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _dp, _vp, _sz, _vp]),
    "pof_dense_workspace_bytes": (_sz, [_i32, _i32, _i64, _i32, _i32, _i32]),
    "pof_dense_linear_filtsmooth": (
        _c.c_int,
        [_i32, _i32, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _dp, _i32, _vp, _sz,
         _vp],
    ),
    "pof_linearize": (_c.c_int, [_i32, _i64, _i32, _i32, _i32, _vp, _f64, _vp, _vp, _vp, _vp]),
    "pof_sequential_linear_filtsmooth": (
        _c.c_int,
        [_i32, _i64, _i32, _i32, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _dp, _vp],
    ),
    "pof_sequential_eks": (
        _c.c_int,
        [_i32, _i64, _i32, _i32, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _dp, _vp],
    ),
    "pof_ieks_solve": (
        _c.c_int,
        [_i32, _i64, _i32, _i32, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _i32, _dp, _vp, _sz, _vp],
    ),
    "pof_ieks_sequential_workspace_bytes": (_sz, [_i32, _i64, _i32, _i32]),
    "pof_ieks_solve_sequential": (
        _c.c_int,
        [_i32, _i64, _i32, _i32, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _i32, _dp, _vp, _sz, _vp],
    ),
    "pof_ieks_mixed_workspace_bytes": (_sz, [_i64, _i32, _i32]),
    "pof_ieks_solve_mixed": (
        _c.c_int,
        [_i64, _i32, _i32, _i32, _vp, _f64, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _f64, _f64, _i64, _i32, _dp, _vp, _sz,
         _vp],
    ),
    "pof_checks_compiled": (_c.c_int, []),
    "pof_checks_read": (_c.c_int, [_vp, _i32]),
    "pof_profile_enable": (None, [_i32]),
    "pof_profile_read": (_c.c_int, [_vp, _vp, _i32, _i32]),
    "pof_fp64_probe": (_c.c_int, [_i64, _i32, _i32, _dp, _vp]),
    "pof_recip_check": (_c.c_int, [_i64, _dp, _dp, _dp, _vp]),
    "pof_batch_workspace_bytes": (_sz, [_i32, _i64, _vp, _i32, _i32, _i32, _i32]),
    "pof_ieks_solve_batch": (
        _c.c_int,
        [_i32, _i64, _vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _i32, _i32, _i32, _dp, _vp,
         _sz, _vp],
    ),
    "pof_server_workspace_bytes": (_sz, [_i32, _i32, _i64, _i64, _sz]),
    "pof_server_create": (_c.c_int, [_i32, _i32, _i64, _i64, _sz, _vp, _vp, _i32, _vp, _sz, _vp]),
    "pof_server_destroy": (_c.c_int, [_vp]),
    "pof_server_mixed_workspace_bytes": (_sz, [_i32, _i32, _i64, _i64, _sz]),
    "pof_server_create_mixed": (_c.c_int, [_i32, _i32, _i64, _i64, _sz, _vp, _vp, _i32, _i64, _f64, _f64, _vp, _sz,
                                           _vp]),
    "pof_server_mixed_info": (_c.c_int, [_vp, _i64, _dp]),
    "pof_server_submit": (_i64, [_vp, _i64, _i32, _vp, _f64, _vp, _vp, _vp, _i64, _f64]),
    "pof_server_launch": (_c.c_int, [_vp, _i64]),
    "pof_server_sync": (_c.c_int, [_vp, _vp]),
    "pof_server_step": (_c.c_int, [_vp, _i64, _vp]),
    "pof_server_cancel": (_c.c_int, [_vp, _i64]),
    "pof_server_poll": (_i64, [_vp, _vp, _i64]),
    "pof_server_fetch": (_c.c_int, [_vp, _i64, _vp, _vp, _dp]),
    "pof_server_stream": (_vp, [_vp]),
    "pof_batch_mixed_workspace_bytes": (_sz, [_i64, _vp, _i32, _i32, _i32, _i32]),
    "pof_ieks_solve_batch_mixed": (
        _c.c_int,
        [_i64, _vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _f64, _f64, _i64, _i32, _i32, _i32,
         _dp, _dp, _vp, _sz, _vp],
    ),
}

PROFILE_KINDS = [
    "linearize", "filt_l0_reduce", "filt_reduce", "filt_top", "filt_down", "filt_l0_down", "filt_finalize",
    "smo_l0_reduce", "smo_reduce", "smo_top", "smo_down", "smo_l0_down", "smo_finalize", "control", "sequential",
]


def profile_enable(on=True):
    lib().pof_profile_enable(int(bool(on)))


def profile_read(reset=True):
    """{kind: (milliseconds, launches)} of the libpof launches since the last reset."""
    n = len(PROFILE_KINDS)
    ms = (ctypes.c_double * n)()
    cnt = (ctypes.c_int64 * n)()
    lib().pof_profile_read(ctypes.cast(ms, ctypes.c_void_p), ctypes.cast(cnt, ctypes.c_void_p), n, int(bool(reset)))
    return {k: (ms[i], cnt[i]) for i, k in enumerate(PROFILE_KINDS)}


def load(path):
    """A libpof build at `path` with the C ABI's signatures set (ctypes)."""
    l = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args
    return l


def lib():
    """The loaded libpof.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PofError(
                "libpof.so not found at %s; build it with `python -m pof._build` "
                "(or __graft_entry__.build())" % LIB_PATH
            )
        _lib = load(LIB_PATH)
    return _lib


def exported_symbols():
    return list(_SIGS)


POF_ERR_BUSY = -7


def check(rc, what=""):
    if rc != POF_OK:
        msg = lib().pof_status_string(rc).decode()
        if rc == -4:
            msg += ": " + lib().pof_last_cuda_error().decode()
        raise PofError("%s failed (%d): %s" % (what or "libpof call", rc, msg))


def dtype_code(dtype):
    if dtype == torch.float64:
        return POF_F64
    if dtype == torch.float32:
        return POF_F32
    raise PofError("unsupported dtype %s" % dtype)


def ptr(t):
    if t is None:
        return None
    if not t.is_cuda:
        raise PofError("libpof needs CUDA tensors (got a %s tensor)" % t.device)
    if not t.is_contiguous():
        raise PofError("libpof needs contiguous tensors")
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def workspace(nbytes, device):
    return torch.empty(int(nbytes), dtype=torch.uint8, device=device)


def solve_status(code):
    """Name of an info[I_STATUS] value ("converged", "maxiters", "nonfinite",
    "cancelled")."""
    return SOLVE_STATUS.get(int(code), "unknown")


def shape_supported(D, d):
    return bool(lib().pof_shape_supported(int(D), int(d)))
