"""Parallel square-root filter (pof/parallel_filtsmooth/filter.py)."""

from . import _call


def linear_noiseless_filtering(x0, transition_models, observation_models):
    """Filtered states of a linear model with exact observations
    (pof/parallel_filtsmooth/filter.py:18-47), computed in libpof with the
    chunked associative scan.  Returns (MVNSqrt, nll, obj, ssq)."""
    out, nll, obj, ssq, _ = _call.filtsmooth("filter", x0, transition_models, observation_models)
    return out, nll, obj, ssq
