"""Argument marshalling for the libpof filter/smoother entry points."""

import torch

from .. import _lib
from ..utils import MVNSqrt


def _contig(t, dtype, device):
    return t.to(device=device, dtype=dtype).contiguous()


def transitions(dtm, n, D, dtype, device):
    """(F, QL, stride): one shared (D, D) pair or per-step (n, D, D) stacks."""
    F, QL = dtm
    if F.dim() == 2:
        return _contig(F, dtype, device), _contig(QL, dtype, device), 0
    if F.dim() == 3 and F.stride(0) == 0 and QL.stride(0) == 0:
        # one (D, D) pair broadcast over the steps (as set_up_solver builds it)
        return _contig(F[0], dtype, device), _contig(QL[0], dtype, device), 0
    if F.shape != (n, D, D) or QL.shape != (n, D, D):
        raise ValueError("transition models must be (n, D, D) or (D, D); got %s, %s" % (tuple(F.shape), tuple(QL.shape)))
    return _contig(F, dtype, device), _contig(QL, dtype, device), D * D


def observations(dom, n, D, dtype, device):
    H, c, R = dom
    d = c.shape[-1]
    if H.shape != (n, d, D) or c.shape != (n, d):
        raise ValueError("observation models must be H (n, d, D), b (n, d); got %s, %s" % (tuple(H.shape), tuple(c.shape)))
    H = _contig(H, dtype, device)
    c = _contig(c, dtype, device)
    if R is None:
        return H, c, None, 0, d
    R = _contig(R, dtype, device)
    if R.dim() == 2:
        return H, c, R, 0, d
    if R.shape != (n, d, d):
        raise ValueError("cholR must be (n, d, d) or (d, d)")
    return H, c, R, d * d, d


DENSE_WHICH = {"filter": 0, "filtsmooth": 1, "smoothing": 2}


def filtsmooth(which, x0: MVNSqrt, dtm, dom, stream=None, dense_chunks=None):
    """which = "filtsmooth" | "filter": run the chunked parallel pass in libpof.
    dense_chunks (an int >= 0): run libpof's dense path
    (pof_dense_linear_filtsmooth) with that many chunks (0: its default),
    whatever D is; None: libpof picks (the dense path for uncompiled shapes
    with D >= 32)."""
    m0 = x0.mean
    device = m0.device if m0.is_cuda else torch.device("cuda", torch.cuda.current_device())
    dtype = m0.dtype if m0.dtype in (torch.float64, torch.float32) else torch.float64
    n = dom[0].shape[0]
    D = m0.shape[-1]
    F, QL, fts = transitions(dtm, n, D, dtype, device)
    H, c, R, rs, d = observations(dom, n, D, dtype, device)
    m0 = _contig(m0, dtype, device)
    L0 = _contig(x0.chol, dtype, device)
    means = torch.empty((n + 1, D), dtype=dtype, device=device)
    chols = torch.empty((n + 1, D, D), dtype=dtype, device=device)
    scal = torch.zeros(_lib.S_COUNT, dtype=torch.float64, device=device)
    lib = _lib.lib()
    code = _lib.dtype_code(dtype)
    if dense_chunks is not None:
        wh = DENSE_WHICH[which]
        wsb = lib.pof_dense_workspace_bytes(code, wh, n, D, d, int(dense_chunks))
        ws = _lib.workspace(wsb, device)
        rc = lib.pof_dense_linear_filtsmooth(wh, code, n, D, d, _lib.ptr(m0), _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL),
                                             fts, _lib.ptr(H), _lib.ptr(c), _lib.ptr(R), rs, _lib.ptr(means),
                                             _lib.ptr(chols), _lib.ptr(scal), int(dense_chunks), _lib.ptr(ws), wsb,
                                             _lib.stream_handle(stream))
        _lib.check(rc, "pof_dense_linear_filtsmooth")
        return MVNSqrt(means, chols), scal[_lib.S_NLL], scal[_lib.S_OBJ], scal[_lib.S_SSQ], scal
    wsb = lib.pof_filtsmooth_workspace_bytes(code, n, D, d)
    ws = _lib.workspace(wsb, device)
    fn = lib.pof_linear_filtsmooth if which == "filtsmooth" else lib.pof_linear_noiseless_filtering
    rc = fn(code, n, D, d, _lib.ptr(m0), _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL), fts, _lib.ptr(H), _lib.ptr(c),
            _lib.ptr(R), rs, _lib.ptr(means), _lib.ptr(chols), _lib.ptr(scal), _lib.ptr(ws), wsb,
            _lib.stream_handle(stream))
    _lib.check(rc, "pof_linear_%s" % which)
    return MVNSqrt(means, chols), scal[_lib.S_NLL], scal[_lib.S_OBJ], scal[_lib.S_SSQ], scal


def smoothing(dtm, filt: MVNSqrt, stream=None, dense_chunks=None):
    fm, fL = filt
    device = fm.device
    dtype = fm.dtype
    N, D = fm.shape
    n = N - 1
    F, QL, fts = transitions(dtm, n, D, dtype, device)
    fm = _contig(fm, dtype, device)
    fL = _contig(fL, dtype, device)
    means = torch.empty_like(fm)
    chols = torch.empty_like(fL)
    scal = torch.zeros(_lib.S_COUNT, dtype=torch.float64, device=device)
    lib = _lib.lib()
    code = _lib.dtype_code(dtype)
    d = 1  # the smoother's workspace does not depend on d
    if dense_chunks is not None:
        wsb = lib.pof_dense_workspace_bytes(code, 2, n, D, d, int(dense_chunks))
        ws = _lib.workspace(wsb, device)
        rc = lib.pof_dense_linear_filtsmooth(2, code, n, D, d, _lib.ptr(fm), _lib.ptr(fL), _lib.ptr(F), _lib.ptr(QL),
                                             fts, None, None, None, 0, _lib.ptr(means), _lib.ptr(chols),
                                             _lib.ptr(scal), int(dense_chunks), _lib.ptr(ws), wsb,
                                             _lib.stream_handle(stream))
        _lib.check(rc, "pof_dense_linear_filtsmooth")
        return MVNSqrt(means, chols), scal[_lib.S_OBJ]
    wsb = lib.pof_filtsmooth_workspace_bytes(code, n, D, d)
    ws = _lib.workspace(wsb, device)
    rc = lib.pof_smoothing(code, n, D, _lib.ptr(F), _lib.ptr(QL), fts, _lib.ptr(fm), _lib.ptr(fL), _lib.ptr(means),
                           _lib.ptr(chols), _lib.ptr(scal), _lib.ptr(ws), wsb, _lib.stream_handle(stream))
    _lib.check(rc, "pof_smoothing")
    return MVNSqrt(means, chols), scal[_lib.S_OBJ]
