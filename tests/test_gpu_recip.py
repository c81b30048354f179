"""The double reciprocal and reciprocal square root of the kernels' reflector
scalars (one third-order correction of a single-precision seed, csrc/pof_linalg.cuh)
against IEEE division and square root: within 2 units in the last place
over the whole exponent range the kernels meet, and the IEEE results for
the arguments they hand over (zero, subnormal, huge)."""

import numpy as np
import pytest
import torch

from pof import _lib

pytestmark = pytest.mark.gpu


def test_recip_accuracy():
    rng = np.random.default_rng(0)
    x = np.concatenate([
        rng.uniform(1.0, 2.0, 20000) * np.exp2(rng.integers(-990, 990, 20000)),
        -rng.uniform(1.0, 2.0, 5000) * np.exp2(rng.integers(-990, 990, 5000)),
        np.array([1.0, 2.0, 4.0, 0.5, 3.0, 1e-300, 1e300, 5e-324, 1.7976931348623157e308]),
    ])
    xt = torch.as_tensor(x, device="cuda")
    r = torch.empty_like(xt)
    q = torch.empty_like(xt)
    _lib.check(_lib.lib().pof_recip_check(len(x), _lib.ptr(xt), _lib.ptr(r), _lib.ptr(q), _lib.stream_handle()))
    r, q = r.cpu().numpy(), q.cpu().numpy()
    ref_r = 1.0 / x
    ok = np.isfinite(ref_r) & (ref_r != 0)
    ulp = np.abs(r[ok] - ref_r[ok]) / np.spacing(np.abs(ref_r[ok]))
    assert ulp.max() <= 2.0, ulp.max()
    pos = x > 0
    ref_q = 1.0 / np.sqrt(x[pos])
    ulq = np.abs(q[pos] - ref_q) / np.spacing(ref_q)
    assert ulq.max() <= 2.0, ulq.max()
    assert (q[~pos] == 0).all()
