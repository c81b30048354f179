"""JAX's associative scan, restated for tuples of stacked NumPy arrays.

The reference calls ``jax.lax.associative_scan`` (jax 0.3.23, pinned in
``poetry.lock:467-497``) at ``pof/parallel_filtsmooth/filter.py:35`` and
``pof/parallel_filtsmooth/smoother.py:15-17``.  JAX is absent here, so its
published recursion is restated: combine adjacent pairs (0,1), (2,3), ...;
scan the reduced sequence recursively (it holds the results at odd
positions); combine those with the original elements at even positions >= 2;
position 0 is the first element itself; interleave.  ``reverse=True`` reverses
the inputs and the outputs, so ``fn(a, b)`` always receives the element that is
earlier in the (possibly reversed) scan order as ``a``.

The combine order (which pairs are formed at which level) follows JAX exactly,
so the rounding of this oracle follows the reference's tree, not a sequential
left fold.
"""

import numpy as np


def _sl(elems, start, stop, step=1):
    return tuple(e[start:stop:step] for e in elems)


def _interleave(even, odd):
    n = even.shape[0] + odd.shape[0]
    out = np.empty((n,) + even.shape[1:], dtype=np.result_type(even, odd))
    out[0::2] = even
    out[1::2] = odd
    return out


def associative_scan(fn, elems, reverse=False):
    """Inclusive scan of ``elems`` (a tuple of arrays stacked on axis 0)."""
    elems = tuple(np.asarray(e) for e in elems)
    if reverse:
        elems = tuple(e[::-1] for e in elems)

    def _scan(el):
        n = el[0].shape[0]
        if n < 2:
            return el
        # pairs (0,1), (2,3), ...: slice 0:-1:2 and 1::2
        reduced = fn(_sl(el, 0, -1, 2), _sl(el, 1, None, 2))
        odd = _scan(reduced)
        left = _sl(odd, 0, -1) if n % 2 == 0 else odd
        right = _sl(el, 2, None, 2)
        if right[0].shape[0] > 0:
            even = fn(left, right)
            even = tuple(np.concatenate([e[0:1], r]) for e, r in zip(el, even))
        else:
            even = tuple(e[0:1] for e in el)
        return tuple(_interleave(e, o) for e, o in zip(even, odd))

    out = _scan(elems)
    if reverse:
        out = tuple(e[::-1] for e in out)
    return out


def sequential_scan(fn, elems, reverse=False):
    """Left fold with the same operator (a different rounding order)."""
    elems = tuple(np.asarray(e) for e in elems)
    if reverse:
        elems = tuple(e[::-1] for e in elems)
    n = elems[0].shape[0]
    outs = [tuple(e[0] for e in elems)]
    for i in range(1, n):
        a = tuple(x[None] for x in outs[-1])
        b = tuple(e[i : i + 1] for e in elems)
        outs.append(tuple(x[0] for x in fn(a, b)))
    out = tuple(np.stack([o[j] for o in outs]) for j in range(len(elems)))
    if reverse:
        out = tuple(e[::-1] for e in out)
    return out
