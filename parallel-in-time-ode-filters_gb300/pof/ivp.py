"""Initial value problems (pof/ivp.py), as torch vector fields.

Each constructor returns an ``InitialValueProblem`` whose ``f(t, y)`` is a
torch function (usable with ``torch.func`` transforms, on any device) and
carries ``f.pof_field = (name, params)``: the solver recognises the field and
linearizes it on the device with its analytic Jacobian instead of
``torch.func.jacfwd``.
"""

from typing import Callable, NamedTuple

import torch


class InitialValueProblem(NamedTuple):
    """Same fields as ``tornadox.ivp.InitialValueProblem`` (used at pof/ivp.py:14)."""

    f: Callable
    t0: float
    tmax: float
    y0: torch.Tensor

    @property
    def t_span(self):
        return (self.t0, self.tmax)

    @property
    def dimension(self):
        return self.y0.shape[0]


def _tag(f, name, params):
    f.pof_field = (name, tuple(float(p) for p in params))
    return f


def _y0(y0, default):
    return torch.as_tensor(default if y0 is None else y0, dtype=torch.float64)


def logistic(t0=0.0, tmax=10.0, y0=None, r=1.0):
    """y' = r y (1 - y), y0 = 0.01 (pof/ivp.py:7-14 with r = 1)."""

    def f(t, y):
        return r * y * (1 - y)

    return InitialValueProblem(_tag(f, "logistic", (r,)), t0, tmax, _y0(y0, [0.01]))


def lotkavolterra(t0=0.0, tmax=7, y0=None, p=None):
    """pof/ivp.py:17-31."""
    p = (1.5, 1.0, 3.0, 1.0) if p is None else tuple(p)
    a, b, c, d = p

    def f(t, Y):
        return torch.stack([a * Y[0] - b * Y[0] * Y[1], -c * Y[1] + d * Y[0] * Y[1]])

    return InitialValueProblem(_tag(f, "lotkavolterra", p), t0, tmax, _y0(y0, [1.0, 1.0]))


def vanderpol(t0=0.0, tmax=6.3, y0=None, stiffness_constant=1e1):
    """pof/ivp.py:34-41."""
    mu = stiffness_constant

    def f(t, Y):
        return torch.stack([Y[1], mu * ((1.0 - Y[0] ** 2) * Y[1] - Y[0])])

    return InitialValueProblem(_tag(f, "vanderpol", (mu,)), t0, tmax, _y0(y0, [2.0, 0.0]))


def fitzhughnagumo(t0=0.0, tmax=100.0, y0=None, p=None):
    """pof/ivp.py:44-60: (a, b, 1/tau, I) = (0.7, 0.8, 1/12.5, 0.5)."""
    p = (0.7, 0.8, 1 / 12.5, 0.5) if p is None else tuple(p)
    a, b, tinv, l = p

    def f(t, Y):
        v, w = Y[0], Y[1]
        return torch.stack([v - (v**3) / 3 - w + l, tinv * (v + a - b * w)])

    return InitialValueProblem(_tag(f, "fitzhughnagumo", p), t0, tmax, _y0(y0, [1.0, 1.0]))


def fhn_classic(t0=0.0, tmax=100.0, y0=None, a=0.2, b=0.2, c=3.0):
    """FitzHugh-Nagumo in (a, b, c) form: y1' = c (y1 - y1^3/3 + y2),
    y2' = -(y1 - a + b y2) / c, y0 = (-1, 1)."""

    def f(t, Y):
        return torch.stack([c * (Y[0] - Y[0] ** 3 / 3 + Y[1]), -(Y[0] - a + b * Y[1]) / c])

    return InitialValueProblem(_tag(f, "fhn_classic", (a, b, c)), t0, tmax, _y0(y0, [-1.0, 1.0]))


def rober(t0=0.0, tmax=1e11, y0=None, p=None):
    """pof/ivp.py:63-79."""
    p = (0.04, 3e7, 1e4) if p is None else tuple(p)
    k1, k2, k3 = p

    def f(t, Y):
        y1, y2, y3 = Y[0], Y[1], Y[2]
        return torch.stack([-k1 * y1 + k3 * y2 * y3, k1 * y1 - k2 * y2**2 - k3 * y2 * y3, k2 * y2**2])

    return InitialValueProblem(_tag(f, "rober", p), t0, tmax, _y0(y0, [1.0, 0.0, 0.0]))


def rigid_body(t0=0.0, tmax=20.0, y0=None, p=None):
    """pof/ivp.py:82-90."""
    p = (-2.0, 1.25, -0.5) if p is None else tuple(p)

    def f(t, y):
        return torch.stack([p[0] * y[1] * y[2], p[1] * y[0] * y[2], p[2] * y[0] * y[1]])

    return InitialValueProblem(_tag(f, "rigid_body", p), t0, tmax, _y0(y0, [1.0, 0.0, 0.9]))


def seir(t0=0.0, tmax=200.0, y0=None, p=None):
    """pof/ivp.py:93-108."""
    y0 = _y0(y0, [998.0, 1.0, 1.0, 1.0])
    p = (0.3, 0.3, 0.1, float(y0.sum())) if p is None else tuple(p)

    def f(t, y):
        return torch.stack(
            [
                -p[1] * y[0] * y[2] / p[3],
                p[1] * y[0] * y[2] / p[3] - p[0] * y[1],
                p[0] * y[1] - p[2] * y[2],
                p[2] * y[2],
            ]
        )

    return InitialValueProblem(_tag(f, "seir", p), t0, tmax, y0)


def threebody(t0=0.0, tmax=17.0652165601579625588917206249, y0=None, p=None):
    """pof/ivp.py:111-126."""
    p = (0.012277471,) if p is None else tuple(p)
    mu = p[0]
    mp = 1.0 - mu

    def f(t, y):
        D1 = torch.sqrt((y[0] + mu) ** 2 + y[1] ** 2) ** 3.0
        D2 = torch.sqrt((y[0] - mp) ** 2 + y[1] ** 2) ** 3.0
        du0p = y[0] + 2 * y[3] - mp * (y[0] + mu) / D1 - mu * (y[0] - mp) / D2
        du1p = y[1] - 2 * y[2] - mp * y[1] / D1 - mu * y[1] / D2
        return torch.stack([y[2], y[3], du0p, du1p])

    y0 = _y0(y0, [0.994, 0.0, 0.0, -2.00158510637908252240537862224])
    return InitialValueProblem(_tag(f, "threebody", p), t0, tmax, y0)


def henonheiles(t0=0.0, tmax=100.0, y0=None, p=None):
    """pof/ivp.py:137-152."""
    p = 1.0 if p is None else p

    def f(t, y):
        return torch.stack([y[2], y[3], -y[0] - 2 * p * y[0] * y[1], -y[1] - p * (y[0] ** 2 - y[1] ** 2)])

    return InitialValueProblem(_tag(f, "henonheiles", (p,)), t0, tmax, _y0(y0, [0.5, 0.0, 0.0, 0.1]))


def fhn_reaction_diffusion(t0=0.0, tmax=20.0, y0=None, cells=64, a=0.2, b=0.2, c=3.0, kv=0.5, kw=0.05, amp=0.5):
    """Method-of-lines FitzHugh-Nagumo reaction-diffusion system on a periodic
    1-D grid of `cells` cells (d = 2 cells; not in the reference's pof.ivp):
    v_k' = c (v_k - v_k^3 / 3 + w_k) + kv (v_{k-1} - 2 v_k + v_{k+1}),
    w_k' = -(v_k - a + b w_k) / c + kw (w_{k-1} - 2 w_k + w_{k+1}),
    kv, kw the diffusion coefficients over the squared cell width.  Default
    initial state: v = -1 + amp sin(2 pi k / cells), w = 1 (the FitzHugh-Nagumo
    y0 = (-1, 1) with a sine perturbation)."""
    m = int(cells)
    if y0 is None:
        k = torch.arange(m, dtype=torch.float64)
        y0 = torch.cat([-1.0 + amp * torch.sin(2.0 * torch.pi * k / m), torch.ones(m, dtype=torch.float64)])

    def lap(u):
        return torch.roll(u, 1, -1) - 2.0 * u + torch.roll(u, -1, -1)

    def f(t, Y):
        v, w = Y[..., :m], Y[..., m:]
        dv = c * (v - v * v * v / 3.0 + w) + kv * lap(v)
        dw = -(v - a + b * w) / c + kw * lap(w)
        return torch.cat([dv, dw], -1)

    return InitialValueProblem(_tag(f, "fhn_rd", (a, b, c, kv, kw)), t0, tmax, _y0(y0, None))
