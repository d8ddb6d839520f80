"""``jax.numpy`` on NumPy (test infrastructure; see ``jax/__init__.py``).

Every attribute is NumPy's; functions are wrapped so that array results are
:class:`ndarray` views, which carry JAX's functional update syntax
``x.at[idx].set(v)`` (a copy with ``idx`` replaced), ``.add``/``.mul``/
``.multiply`` (unbuffered, so repeated indices accumulate as in JAX's
scatter-add) and ``.get``.
"""

from __future__ import annotations

import functools as _ft
import types as _types

import numpy as _np


def _clamp_one(i, n):
    if isinstance(i, (bool, _np.bool_)) or isinstance(i, slice) or i is None or i is Ellipsis:
        return i
    if isinstance(i, (int, _np.integer)):
        i = int(i)
        if i < 0:
            i += n
        return min(max(i, 0), n - 1)
    if isinstance(i, _np.ndarray) and i.dtype.kind in "iu":
        j = _np.where(i < 0, i + n, i)
        return _np.clip(j, 0, n - 1).view(_np.ndarray)
    return i


def _clamp_index(shape, idx):
    """JAX gathers clamp out-of-range integer indices instead of raising."""
    if not isinstance(idx, tuple):
        idx = (idx,)
    if any(isinstance(i, _np.ndarray) and i.dtype == bool for i in idx):
        return tuple(_plain(idx))
    n_axes = sum(0 if (i is None or i is Ellipsis) else 1 for i in idx)
    out = []
    ax = 0
    for i in idx:
        if i is Ellipsis:
            ax += len(shape) - n_axes
            out.append(i)
            continue
        if i is None:
            out.append(i)
            continue
        out.append(_clamp_one(_plain(i), shape[ax]) if ax < len(shape) else i)
        ax += 1
    return tuple(out)


class ndarray(_np.ndarray):
    """np.ndarray with the jax.Array methods that the reference calls, and
    JAX's clamping of out-of-range integer indices on reads."""

    def __getitem__(self, idx):
        return super().__getitem__(_clamp_index(self.shape, idx))

    def __iter__(self):
        if self.ndim == 0:
            raise TypeError("iteration over a 0-d array")
        get = super().__getitem__
        return (get(i) for i in range(self.shape[0]))

    @property
    def at(self):
        return _At(self)

    def delete(self):
        """JAX frees the device buffer; NumPy's garbage collector does it here."""

    def block_until_ready(self):
        return self

    def devices(self):
        import jax

        return {jax.devices()[0]}


class _At:
    __slots__ = ("arr",)

    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtRef(self.arr, idx)


def _plain(idx):
    if isinstance(idx, tuple):
        return tuple(_plain(i) for i in idx)
    if isinstance(idx, ndarray):
        return idx.view(_np.ndarray)
    return idx


class _AtRef:
    __slots__ = ("arr", "idx")

    def __init__(self, arr, idx):
        self.arr = arr
        self.idx = _plain(idx)

    def get(self, **kw):
        return _wrap(_np.asarray(self.arr)[self.idx])

    def set(self, values, **kw):
        out = _np.array(self.arr, copy=True)
        out[self.idx] = _np.asarray(values)
        return _wrap(out)

    def _ufunc_at(self, uf, values):
        out = _np.array(self.arr, copy=True)
        uf.at(out, self.idx, _np.asarray(values))
        return _wrap(out)

    def add(self, values, **kw):
        return self._ufunc_at(_np.add, values)

    def multiply(self, values, **kw):
        return self._ufunc_at(_np.multiply, values)

    mul = multiply

    def min(self, values, **kw):
        return self._ufunc_at(_np.minimum, values)

    def max(self, values, **kw):
        return self._ufunc_at(_np.maximum, values)


def _wrap(x):
    if isinstance(x, ndarray):
        return x
    if isinstance(x, _np.ndarray):
        return x.view(ndarray)
    if isinstance(x, tuple):
        return tuple(_wrap(e) for e in x)
    if isinstance(x, list):
        return [_wrap(e) for e in x]
    return x


def _wrap_fn(fn):
    @_ft.wraps(fn)
    def call(*a, **k):
        k.pop("device", None)
        return _wrap(fn(*a, **k))

    return call


def _wrap_module(mod, name):
    out = _types.ModuleType(name)
    for k in dir(mod):
        if k.startswith("__"):
            continue
        v = getattr(mod, k)
        if callable(v) and not isinstance(v, type):
            v = _wrap_fn(v)
        setattr(out, k, v)
    return out


linalg = _wrap_module(_np.linalg, "jax.numpy.linalg")
fft = _wrap_module(_np.fft, "jax.numpy.fft")


def array(obj, dtype=None, copy=True, **kw):
    kw.pop("device", None)
    if isinstance(obj, (list, tuple)):
        obj = [_np.asarray(o) if isinstance(o, _np.ndarray) else o for o in obj]
    return _wrap(_np.array(obj, dtype=dtype, copy=True, **kw))


def asarray(obj, dtype=None, **kw):
    kw.pop("device", None)
    return _wrap(_np.asarray(obj, dtype=dtype, **kw))


_cache: dict = {}


def __getattr__(name):
    if name in _cache:
        return _cache[name]
    v = getattr(_np, name)
    if callable(v) and not isinstance(v, type):
        v = _wrap_fn(v)
    _cache[name] = v
    return v
