"""Convergence criterion of the IEKS loop (pof/convergence_criteria.py)."""

import torch


def crit(obj, obj_old, nll, nll_old, states, states_old, *, rtol=1e-6, atol=1e-9):
    """True when NaN appeared, the objective stalled (isclose(obj_old, obj,
    rtol, atol)) or every mean is isclose(old, new, rtol=1e-13, atol=1e-8)
    (pof/convergence_criteria.py:4-13).  Returns a 0-dim bool tensor."""
    obj = torch.as_tensor(obj, dtype=torch.float64)
    obj_old = torch.as_tensor(obj_old, dtype=torch.float64, device=obj.device)
    nll = torch.as_tensor(nll, dtype=torch.float64, device=obj.device)
    isnan = torch.isnan(obj) | torch.isnan(nll)
    obj_converged = torch.isclose(obj_old, obj, rtol=rtol, atol=atol)
    means, means_old = states.mean, states_old.mean
    means_converged = torch.isclose(means_old, means, rtol=1e-13, atol=1e-8).all()
    converged = obj_converged | means_converged.to(obj_converged.device)
    return isnan | converged
