"""Sequential square-root filter and smoother (pof/sequential_filtsmooth):
the reference's sequential twin, run step after step by libpof on the GPU."""

from .filter import extended_kalman_filter, linear_noiseless_filter, _sqrt_predict, _sqrt_update  # noqa: F401
from .smoother import smoothing  # noqa: F401
from . import _call


def filtsmooth(x0, linear_transitions, continuous_observation_model):
    """EKF (linearizing at each predicted mean) + RTS smoother
    (pof/sequential_filtsmooth/__init__.py:5-10).  Returns (MVNSqrt, nll, obj, ssq)
    where nll is the summed log-likelihood with the sequential twin's sign.
    Built-in fields run both passes in libpof's sequential kernel; other
    torch fields run the EKF step by step in torch and the smoother in
    libpof."""
    if getattr(continuous_observation_model, "field", None) is None:
        out, nll, ssq = extended_kalman_filter(x0, linear_transitions, continuous_observation_model)
        out, obj = smoothing(linear_transitions, out)
        return out, nll, obj, ssq
    return _call.sequential(x0, linear_transitions, om=continuous_observation_model)


def linear_filtsmooth(x0, linear_transitions, linear_observations):
    """Linear filter + RTS smoother (pof/sequential_filtsmooth/__init__.py:13-16)."""
    return _call.sequential(x0, linear_transitions, dom=linear_observations)
