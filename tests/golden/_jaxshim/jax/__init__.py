"""A NumPy stand-in for the small part of the ``jax`` API that meliao/jaxhps
uses.  TEST INFRASTRUCTURE ONLY: ``tests/golden/make_fixtures.py`` puts this
folder on ``sys.path`` so that the unmodified reference package
(``src/jaxhps``) imports and runs on the CPU in a container without ``jax``,
and writes its outputs as golden fixtures.  Nothing in the product package,
``bench.py`` or the tests' run time imports it.

What it provides, and how it maps to NumPy:

* ``jax.numpy``: every NumPy function, with array results viewed as
  :class:`jax.numpy.ndarray` (an ``np.ndarray`` subclass that adds the
  functional update ``x.at[idx].set/add/mul/multiply/get``, ``delete`` and
  ``block_until_ready``).  FP64 is NumPy's default, which is what the
  reference asks for with ``jax_enable_x64``.
* ``jax.vmap``: a Python loop over the mapped axis, outputs stacked.
* ``jax.jit``: the identity (static arguments are plain Python values here).
* ``jax.lax.{fori_loop, cond, switch, dynamic_slice}``: their documented
  semantics on concrete values (``dynamic_slice`` clamps its start indices
  as XLA's DynamicSlice does).
* ``jax.tree_util`` / ``jax.tree``: a pytree registry with ``tree_flatten``
  (tree definitions compare equal when their node types and auxiliary data
  do) and ``tree.map``.
* ``jax.devices`` / ``device_put``: one CPU device; placement is a no-op.

The arithmetic therefore is NumPy's (LAPACK ``gesv``-based ``inv``, BLAS
products) where the reference would run XLA's CPU kernels: the two agree to
rounding, which is the level at which the fixtures are compared.
"""

from __future__ import annotations

import numpy as _np

from . import numpy  # noqa: F401  (jax.numpy)
from . import lax, tree, tree_util, typing, sharding, debug  # noqa: F401
from .numpy import ndarray as Array, _wrap

__version__ = "0.0-numpy-stand-in"


class Device:
    """One CPU device."""

    platform = "cpu"
    device_kind = "cpu"
    id = 0

    def memory_stats(self):
        return {"bytes_limit": 0}

    def __repr__(self):
        return "CpuDevice(id=0)"


_CPU = Device()
Dtype = _np.dtype


def devices(backend=None):
    if backend not in (None, "cpu"):
        raise RuntimeError(f"Unknown backend {backend}")
    return [_CPU]


def local_devices(*a, **k):
    return [_CPU]


def device_put(x, device=None, *a, **k):
    if isinstance(x, (list, tuple)):
        return type(x)(device_put(e) for e in x)
    if isinstance(x, _np.ndarray):
        return _wrap(x)
    return x


def block_until_ready(x):
    return x


class _Config:
    def update(self, name, value):
        if name == "jax_enable_x64" and not value:
            raise NotImplementedError("the stand-in computes in FP64 only")

    def __getattr__(self, name):
        return None


config = _Config()


def jit(fun=None, **kwargs):
    """Identity: arguments are concrete, so compilation changes nothing."""
    if fun is None:
        return lambda f: f
    return fun


def _axes_for(axes, n):
    if isinstance(axes, (tuple, list)):
        if len(axes) != n:
            raise ValueError("vmap in_axes length does not match the arguments")
        return list(axes)
    return [axes] * n


def vmap(fun, in_axes=0, out_axes=0):
    """Loop over the mapped axis and stack the results (jax.vmap semantics on
    concrete arrays: arguments with axis ``None`` are passed unchanged)."""

    def mapped(*args):
        axes = _axes_for(in_axes, len(args))
        size = None
        for a, ax in zip(args, axes):
            if ax is None:
                continue
            for leaf in tree_util.tree_leaves(a):
                n = _np.shape(leaf)[ax]
                if size is None:
                    size = n
                elif n != size:
                    raise ValueError("vmap got inconsistent sizes for the mapped axis")
        if size is None:
            raise ValueError("vmap needs at least one mapped argument")

        def take(a, ax, i):
            if ax is None:
                return a
            return tree_util.tree_map(lambda x: _wrap(_np.take(_np.asarray(x), i, axis=ax)), a)

        outs = [fun(*[take(a, ax, i) for a, ax in zip(args, axes)]) for i in range(size)]
        return _stack_tree(outs, out_axes)

    return mapped


def _stack_tree(outs, out_axes):
    first = outs[0]
    if isinstance(first, (tuple, list)):
        oax = out_axes if isinstance(out_axes, (tuple, list)) else [out_axes] * len(first)
        parts = [_stack_tree([o[k] for o in outs], oax[k]) for k in range(len(first))]
        return type(first)(parts) if isinstance(first, tuple) else parts
    if isinstance(first, dict):
        return {k: _stack_tree([o[k] for o in outs], out_axes) for k in first}
    if first is None:
        return None
    return _wrap(_np.stack([_np.asarray(o) for o in outs], axis=out_axes))
