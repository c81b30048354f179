"""Argument marshalling for libpof's sequential entry points."""

import torch

from .. import _lib
from ..parallel_filtsmooth._call import _contig, observations, transitions
from ..utils import MVNSqrt


def field_params(field, dtype, device):
    name, params = field
    return _lib.FIELDS[name], torch.tensor(params if params else (0.0,), dtype=dtype, device=device)


def sequential(x0, dtm, dom=None, om=None, smooth=True, stream=None):
    m0 = x0.mean
    device = m0.device
    dtype = m0.dtype
    D = m0.shape[-1]
    F0 = dtm[0]
    n = F0.shape[0] if F0.dim() == 3 else (dom[0].shape[0] if dom is not None else None)
    F, QL, fts = transitions(dtm, n, D, dtype, device)
    m0 = _contig(m0, dtype, device)
    L0 = _contig(x0.chol, dtype, device)
    means = torch.empty((n + 1, D), dtype=dtype, device=device)
    chols = torch.empty((n + 1, D, D), dtype=dtype, device=device)
    scal = torch.zeros(_lib.S_COUNT, dtype=torch.float64, device=device)
    lib = _lib.lib()
    code = _lib.dtype_code(dtype)
    if dom is not None:
        H, c, R, rs, d = observations(dom, n, D, dtype, device)
        rc = lib.pof_sequential_linear_filtsmooth(code, n, D, d, _lib.ptr(m0), _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL),
                                                  fts, _lib.ptr(H), _lib.ptr(c), _lib.ptr(R), rs, int(smooth), _lib.ptr(means),
                                                  _lib.ptr(chols), _lib.ptr(scal), _lib.stream_handle(stream))
        _lib.check(rc, "pof_sequential_linear_filtsmooth")
    else:
        field = getattr(om, "field", None)
        if field is None:
            raise ValueError("libpof's sequential EKF linearizes built-in fields only (pof.ivp); "
                             "pof.sequential_filtsmooth.filtsmooth runs other fields step by step in torch")
        setup = om.setup
        fid, params = field_params(field, dtype, device)
        d = setup["iwp"].wiener_process_dimension
        rc = lib.pof_sequential_eks(code, n, D, d, fid, _lib.ptr(params), float(setup["dt"]), _lib.ptr(m0),
                                    _lib.ptr(L0), _lib.ptr(F), _lib.ptr(QL), fts, int(smooth), _lib.ptr(means), _lib.ptr(chols),
                                    _lib.ptr(scal), _lib.stream_handle(stream))
        _lib.check(rc, "pof_sequential_eks")
    return MVNSqrt(means, chols), scal[_lib.S_NLL], scal[_lib.S_OBJ], scal[_lib.S_SSQ]
