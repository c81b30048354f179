"""Parallel-in-time square-root filter and smoother
(pof/parallel_filtsmooth/__init__.py): entry points backed by libpof."""

from .filter import linear_noiseless_filtering
from .smoother import smoothing
from . import _call


def linear_filtsmooth(x0, linear_transitions, linear_observations):
    """Filter then smoother (pof/parallel_filtsmooth/__init__.py:5-10).

    Returns (MVNSqrt(means (N, D), chols (N, D, D)), nll, obj, ssq): nll and
    ssq of the filter, obj of the smoother, as 0-dim device tensors."""
    out, nll, obj, ssq, _ = _call.filtsmooth("filtsmooth", x0, linear_transitions, linear_observations)
    return out, nll, obj, ssq


__all__ = ["linear_filtsmooth", "linear_noiseless_filtering", "smoothing"]
