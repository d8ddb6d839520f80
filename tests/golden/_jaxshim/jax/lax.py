"""``jax.lax`` control flow on concrete values (test infrastructure; see
``jax/__init__.py``)."""

from __future__ import annotations

import numpy as _np

from .numpy import _wrap


def fori_loop(lower, upper, body_fun, init_val):
    val = init_val
    for i in range(int(lower), int(upper)):
        val = body_fun(i, val)
    return val


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def switch(index, branches, *operands):
    i = min(max(int(index), 0), len(branches) - 1)
    return branches[i](*operands)


def dynamic_slice(operand, start_indices, slice_sizes):
    """XLA DynamicSlice: start indices are clamped so the slice lies inside."""
    x = _np.asarray(operand)
    sl = []
    for s, n, dim in zip(start_indices, slice_sizes, x.shape):
        s = min(max(int(s), 0), dim - int(n))
        sl.append(slice(s, s + int(n)))
    return _wrap(x[tuple(sl)])
