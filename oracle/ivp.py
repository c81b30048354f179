"""The reference's built-in vector fields, plus the two fields of the
benchmark configurations (test infrastructure).

``pof/ivp.py`` wraps each field as a ``tornadox.ivp.InitialValueProblem``
(f, t0, tmax, y0).  Here an ``IVP`` carries ``components`` (a function of a
list of scalars, usable with floats, arrays and ``Taylor`` series), ``y0``,
``t0``, ``tmax``; ``f(t, y)`` evaluates it on arrays.
"""

from typing import Callable, NamedTuple, Optional

import numpy as np

from . import taylor


class IVP(NamedTuple):
    components: Callable
    y0: np.ndarray
    t0: float
    tmax: float
    name: str = ""
    params: tuple = ()
    # optional array forms of the field and its Jacobian (large systems)
    f_array: Optional[Callable] = None
    jac_array: Optional[Callable] = None

    def f(self, t, y):
        if self.f_array is not None:
            return self.f_array(np.asarray(y, float))
        return taylor.evaluate(self.components, y)

    def jac(self, y):
        if self.jac_array is not None:
            return self.jac_array(np.asarray(y, float))
        return taylor.jacobian(self.components, y)

    @property
    def t_span(self):
        return (self.t0, self.tmax)


def logistic(t0=0.0, tmax=10.0, y0=None, r=1.0):
    """``pof/ivp.py:7-14`` (r = 1); the scan-length sweep uses r = 3."""
    y0 = np.array([0.01]) if y0 is None else np.asarray(y0, float)
    return IVP(lambda y: [r * y[0] * (1 - y[0])], y0, t0, tmax, "logistic", (r,))


def lotkavolterra(t0=0.0, tmax=7.0, y0=None, p=None):
    """``pof/ivp.py:17-31``."""
    y0 = np.array([1.0, 1.0]) if y0 is None else np.asarray(y0, float)
    a, b, c, d = (1.5, 1.0, 3.0, 1.0) if p is None else p

    def comp(Y):
        return [a * Y[0] - b * Y[0] * Y[1], -c * Y[1] + d * Y[0] * Y[1]]

    return IVP(comp, y0, t0, tmax, "lotkavolterra", (a, b, c, d))


def vanderpol(t0=0.0, tmax=6.3, y0=None, stiffness_constant=1e1):
    """``pof/ivp.py:34-41``."""
    y0 = np.array([2.0, 0.0]) if y0 is None else np.asarray(y0, float)
    mu = stiffness_constant

    def comp(Y):
        return [Y[1], mu * ((1.0 - Y[0] ** 2) * Y[1] - Y[0])]

    return IVP(comp, y0, t0, tmax, "vanderpol", (mu,))


def fitzhughnagumo(t0=0.0, tmax=100.0, y0=None, p=None):
    """``pof/ivp.py:44-60`` (a, b, 1/tau, I) = (0.7, 0.8, 1/12.5, 0.5)."""
    y0 = np.array([1.0, 1.0]) if y0 is None else np.asarray(y0, float)
    a, b, tinv, l = (0.7, 0.8, 1 / 12.5, 0.5) if p is None else p

    def comp(Y):
        v, w = Y[0], Y[1]
        return [v - (v**3) / 3 - w + l, tinv * (v + a - b * w)]

    return IVP(comp, y0, t0, tmax, "fitzhughnagumo", (a, b, tinv, l))


def fhn_classic(t0=0.0, tmax=100.0, y0=None, a=0.2, b=0.2, c=3.0):
    """FitzHugh-Nagumo in the (a, b, c) form of the benchmark configurations:
    y1' = c (y1 - y1^3/3 + y2), y2' = -(y1 - a + b y2) / c, y0 = (-1, 1)."""
    y0 = np.array([-1.0, 1.0]) if y0 is None else np.asarray(y0, float)

    def comp(Y):
        return [c * (Y[0] - Y[0] ** 3 / 3 + Y[1]), -(Y[0] - a + b * Y[1]) / c]

    return IVP(comp, y0, t0, tmax, "fhn_classic", (a, b, c))


def rober(t0=0.0, tmax=1e11, y0=None, p=None):
    """``pof/ivp.py:63-79``."""
    y0 = np.array([1.0, 0.0, 0.0]) if y0 is None else np.asarray(y0, float)
    k1, k2, k3 = (0.04, 3e7, 1e4) if p is None else p

    def comp(Y):
        y1, y2, y3 = Y[0], Y[1], Y[2]
        return [-k1 * y1 + k3 * y2 * y3, k1 * y1 - k2 * y2**2 - k3 * y2 * y3, k2 * y2**2]

    return IVP(comp, y0, t0, tmax, "rober", (k1, k2, k3))


def rigid_body(t0=0.0, tmax=20.0, y0=None, p=None):
    """``pof/ivp.py:82-90``."""
    y0 = np.array([1.0, 0.0, 0.9]) if y0 is None else np.asarray(y0, float)
    p = (-2.0, 1.25, -0.5) if p is None else p

    def comp(y):
        return [p[0] * y[1] * y[2], p[1] * y[0] * y[2], p[2] * y[0] * y[1]]

    return IVP(comp, y0, t0, tmax, "rigid_body", tuple(p))


def seir(t0=0.0, tmax=200.0, y0=None, p=None):
    """``pof/ivp.py:93-108``."""
    y0 = np.array([998.0, 1.0, 1.0, 1.0]) if y0 is None else np.asarray(y0, float)
    p = (0.3, 0.3, 0.1, float(y0.sum())) if p is None else p

    def comp(y):
        return [
            -p[1] * y[0] * y[2] / p[3],
            p[1] * y[0] * y[2] / p[3] - p[0] * y[1],
            p[0] * y[1] - p[2] * y[2],
            p[2] * y[2],
        ]

    return IVP(comp, y0, t0, tmax, "seir", tuple(p))


def threebody(t0=0.0, tmax=17.0652165601579625588917206249, y0=None, p=None):
    """``pof/ivp.py:111-126``."""
    if y0 is None:
        y0 = np.array([0.994, 0.0, 0.0, -2.00158510637908252240537862224])
    mu = 0.012277471 if p is None else p[0]
    mp = 1.0 - mu

    def comp(y):
        D1 = taylor.sqrt((y[0] + mu) ** 2 + y[1] ** 2) ** 3
        D2 = taylor.sqrt((y[0] - mp) ** 2 + y[1] ** 2) ** 3
        du0p = y[0] + 2 * y[3] - mp * (y[0] + mu) / D1 - mu * (y[0] - mp) / D2
        du1p = y[1] - 2 * y[2] - mp * y[1] / D1 - mu * y[1] / D2
        return [y[2], y[3], du0p, du1p]

    return IVP(comp, np.asarray(y0, float), t0, tmax, "threebody", (mu,))


def henonheiles(t0=0.0, tmax=100.0, y0=None, p=None):
    """``pof/ivp.py:137-152``."""
    y0 = np.array([0.5, 0.0, 0.0, 0.1]) if y0 is None else np.asarray(y0, float)
    p = 1.0 if p is None else p

    def comp(y):
        return [y[2], y[3], -y[0] - 2 * p * y[0] * y[1], -y[1] - p * (y[0] ** 2 - y[1] ** 2)]

    return IVP(comp, y0, t0, tmax, "henonheiles", (p,))



def fhn_reaction_diffusion(t0=0.0, tmax=20.0, y0=None, cells=64, a=0.2, b=0.2, c=3.0, kv=0.5, kw=0.05, amp=0.5):
    """Method-of-lines FitzHugh-Nagumo on a periodic grid of `cells` cells,
    y = (v_0..v_{m-1}, w_0..w_{m-1}) (the reaction-diffusion configuration;
    the reference has no such field):
    v_k' = c (v_k - v_k^3 / 3 + w_k) + kv (v_{k-1} - 2 v_k + v_{k+1}),
    w_k' = -(v_k - a + b w_k) / c + kw (w_{k-1} - 2 w_k + w_{k+1})."""
    m = int(cells)
    if y0 is None:
        k = np.arange(m)
        y0 = np.concatenate([-1.0 + amp * np.sin(2.0 * np.pi * k / m), np.ones(m)])
    y0 = np.asarray(y0, float)

    def comp(Y):
        out = []
        for k in range(m):
            v, w = Y[k], Y[m + k]
            out.append(c * (v - v * v * v / 3.0 + w) + kv * (Y[(k - 1) % m] - 2.0 * v + Y[(k + 1) % m]))
        for k in range(m):
            v, w = Y[k], Y[m + k]
            out.append(-(v - a + b * w) / c + kw * (Y[m + (k - 1) % m] - 2.0 * w + Y[m + (k + 1) % m]))
        return out

    def lap(u):
        return np.roll(u, 1, -1) - 2.0 * u + np.roll(u, -1, -1)

    def f_arr(Y):
        v, w = Y[..., :m], Y[..., m:]
        return np.concatenate([c * (v - v * v * v / 3.0 + w) + kv * lap(v), -(v - a + b * w) / c + kw * lap(w)], -1)

    def jac_arr(Y):
        v = Y[..., :m]
        J = np.zeros(Y.shape[:-1] + (2 * m, 2 * m))
        idx = np.arange(m)
        for r0, kd in ((0, kv), (m, kw)):
            J[..., r0 + idx, r0 + (idx - 1) % m] += kd
            J[..., r0 + idx, r0 + (idx + 1) % m] += kd
            J[..., r0 + idx, r0 + idx] += -2.0 * kd
        J[..., idx, idx] += c * (1.0 - v * v)
        J[..., idx, m + idx] += c
        J[..., m + idx, idx] += -1.0 / c
        J[..., m + idx, m + idx] += -b / c
        return J

    return IVP(comp, y0, t0, tmax, "fhn_rd", (a, b, c, kv, kw), f_arr, jac_arr)
