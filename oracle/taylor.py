"""Truncated Taylor-series arithmetic (test infrastructure).

Used for two things the reference gets from JAX:

* Taylor-mode initialisation (``pof/initialization.py:15-22`` calls
  ``tornadox.init.TaylorMode``, tornadox 0.0.1, absent here).  Its published
  algorithm evaluates the vector field on truncated Taylor series with
  ``jax.experimental.jet`` and returns the exact derivatives
  ``y, y', ..., y^(q)`` at t0.  Restated here with the classic coefficient
  recursions (Griewank & Walther, "Evaluating Derivatives", ch. 13).
* Forward-mode Jacobians (``jax.jacfwd`` in ``pof/observations.py:35-40``):
  order-1 series seeded with unit directions.

A ``Taylor`` holds normalised coefficients ``c[k]`` of ``x(t) = sum c[k] t^k``;
``c`` has shape ``(K+1,) + batch`` so one object carries a batch of series.
"""

import math

import numpy as np


class Taylor:
    __array_priority__ = 1000

    def __init__(self, coeffs):
        self.c = np.asarray(coeffs, dtype=np.float64)

    @property
    def K(self):
        return self.c.shape[0] - 1

    def _lift(self, x):
        if isinstance(x, Taylor):
            return x
        c = np.zeros_like(self.c)
        c[0] = x
        return Taylor(c)

    def __add__(self, o):
        return Taylor(self.c + self._lift(o).c)

    __radd__ = __add__

    def __neg__(self):
        return Taylor(-self.c)

    def __sub__(self, o):
        return Taylor(self.c - self._lift(o).c)

    def __rsub__(self, o):
        return Taylor(self._lift(o).c - self.c)

    def __mul__(self, o):
        if not isinstance(o, Taylor):
            return Taylor(self.c * o)
        a, b = np.broadcast_arrays(self.c, o.c)
        out = np.zeros_like(a)
        for k in range(a.shape[0]):
            for i in range(k + 1):
                out[k] = out[k] + a[i] * b[k - i]
        return Taylor(out)

    __rmul__ = __mul__

    def __truediv__(self, o):
        if not isinstance(o, Taylor):
            return Taylor(self.c / o)
        a, b = np.broadcast_arrays(self.c, o.c)
        qc = np.zeros_like(a)
        for k in range(a.shape[0]):
            s = a[k].copy()
            for i in range(k):
                s = s - qc[i] * b[k - i]
            qc[k] = s / b[0]
        return Taylor(qc)

    def __rtruediv__(self, o):
        return self._lift(o) / self

    def __pow__(self, p):
        if isinstance(p, (int, np.integer)) and p >= 0:
            out = self._lift(1.0)
            for _ in range(int(p)):
                out = out * self
            return out
        # real power: k x0 y_k = sum_{j=1..k} ((p+1) j - k) x_j y_{k-j}
        x = self.c
        y = np.zeros_like(x)
        y[0] = x[0] ** p
        for k in range(1, x.shape[0]):
            s = np.zeros_like(x[0])
            for j in range(1, k + 1):
                s = s + ((p + 1) * j - k) * x[j] * y[k - j]
            y[k] = s / (k * x[0])
        return Taylor(y)


def sqrt(x):
    if isinstance(x, Taylor):
        return x**0.5
    return np.sqrt(x)


def _coef(fi, k, like):
    if isinstance(fi, Taylor):
        return fi.c[k]
    return np.broadcast_to(np.asarray(fi, dtype=np.float64) if k == 0 else 0.0, like.shape)


def taylor_derivatives(components, y0, q):
    """Exact derivatives y^(k)(t0), k = 0..q, of y' = f(y), y(t0) = y0.

    ``components(y)`` maps a sequence of scalars (floats or ``Taylor``) to the
    list of the field's components.  Returns shape (q+1, d): the layout
    tornadox's TaylorMode returns.
    """
    y0 = np.asarray(y0, dtype=np.float64)
    d = y0.shape[0]
    coeffs = np.zeros((q + 1, d))
    coeffs[0] = y0
    for k in range(q):
        ys = [Taylor(coeffs[: k + 1, i]) for i in range(d)]
        fs = components(ys)
        for i in range(d):
            coeffs[k + 1, i] = _coef(fs[i], k, coeffs[0, 0]) / (k + 1)
    return coeffs * np.array([math.factorial(k) for k in range(q + 1)])[:, None]


def jacobian(components, y):
    """Forward-mode Jacobian of ``components`` at ``y`` (shape (..., d)) -> (..., d, d)."""
    y = np.asarray(y, dtype=np.float64)
    d = y.shape[-1]
    J = np.zeros(y.shape + (d,))
    for j in range(d):
        ys = []
        for i in range(d):
            c = np.zeros((2,) + y.shape[:-1])
            c[0] = y[..., i]
            c[1] = 1.0 if i == j else 0.0
            ys.append(Taylor(c))
        fs = components(ys)
        for i in range(d):
            J[..., i, j] = _coef(fs[i], 1, y[..., 0])
    return J


def evaluate(components, y):
    """Plain evaluation of ``components`` at ``y`` (shape (..., d)) -> (..., d)."""
    y = np.asarray(y, dtype=np.float64)
    fs = components([y[..., i] for i in range(y.shape[-1])])
    return np.stack([np.broadcast_to(np.asarray(f, dtype=np.float64), y.shape[:-1]) for f in fs], -1)
