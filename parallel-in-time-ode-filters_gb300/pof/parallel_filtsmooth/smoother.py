"""Parallel square-root smoother (pof/parallel_filtsmooth/smoother.py)."""

from ..utils import MVNSqrt
from . import _call


def smoothing(transition_models, filter_trajectory: MVNSqrt):
    """Smoothed states from filtered ones (pof/parallel_filtsmooth/smoother.py:8-22).
    Returns (MVNSqrt, obj)."""
    assert isinstance(filter_trajectory, MVNSqrt) or len(filter_trajectory) == 2
    return _call.smoothing(transition_models, MVNSqrt(*filter_trajectory))
