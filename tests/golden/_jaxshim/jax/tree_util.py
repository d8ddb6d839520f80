"""``jax.tree_util`` pytree registry (test infrastructure; see
``jax/__init__.py``).  A tree definition is a nested tuple
``(node type, auxiliary data, child definitions)``; two definitions are equal
when their types match and their auxiliary data compare equal element by
element (objects by identity, arrays by value)."""

from __future__ import annotations

import numpy as _np

_REGISTRY: dict = {}


def register_pytree_node(nodetype, flatten_func, unflatten_func):
    _REGISTRY[nodetype] = (flatten_func, unflatten_func)


def _children(x):
    """(children, aux, rebuild) for a container node, or None for a leaf."""
    if isinstance(x, (list, tuple)) and not hasattr(x, "_fields"):
        return list(x), None, (lambda ch, t=type(x): t(ch))
    if isinstance(x, dict):
        keys = sorted(x)
        return [x[k] for k in keys], tuple(keys), (lambda ch, ks=keys: dict(zip(ks, ch)))
    if x is None:
        return [], None, (lambda ch: None)
    reg = _REGISTRY.get(type(x))
    if reg is not None:
        ch, aux = reg[0](x)
        ch = [] if ch is None else list(ch)
        return ch, aux, (lambda c, a=aux, u=reg[1]: u(a, tuple(c)))
    return None


class _AuxKey:
    """Wraps auxiliary data so that == compares arrays by value, objects by identity."""

    __slots__ = ("v",)

    def __init__(self, v):
        self.v = v

    def __eq__(self, other):
        return _aux_eq(self.v, other.v)


def _aux_eq(a, b):
    if isinstance(a, (tuple, list)) and isinstance(b, (tuple, list)):
        return len(a) == len(b) and all(_aux_eq(x, y) for x, y in zip(a, b))
    if isinstance(a, _np.ndarray) or isinstance(b, _np.ndarray):
        return _np.shape(a) == _np.shape(b) and bool(_np.all(_np.asarray(a) == _np.asarray(b)))
    if isinstance(a, (int, float, complex, str, bool, type(None), _np.generic)):
        return bool(a == b)
    return a is b


def _flatten(x, is_leaf, leaves):
    if is_leaf is not None and is_leaf(x):
        leaves.append(x)
        return ("leaf",)
    c = _children(x)
    if c is None:
        leaves.append(x)
        return ("leaf",)
    ch, aux, _ = c
    return (type(x), _AuxKey(aux), tuple(_flatten(e, is_leaf, leaves) for e in ch))


def tree_flatten(tree, is_leaf=None):
    leaves: list = []
    treedef = _flatten(tree, is_leaf, leaves)
    return leaves, treedef


def tree_leaves(tree, is_leaf=None):
    return tree_flatten(tree, is_leaf)[0]


def tree_map(f, tree, *rest, is_leaf=None):
    if is_leaf is not None and is_leaf(tree):
        return f(tree, *rest)
    c = _children(tree)
    if c is None:
        return f(tree, *rest)
    ch, _, rebuild = c
    rest_ch = [_children(r)[0] for r in rest]
    return rebuild([tree_map(f, e, *[r[i] for r in rest_ch], is_leaf=is_leaf) for i, e in enumerate(ch)])
